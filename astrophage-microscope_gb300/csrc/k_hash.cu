// k_hash.cu -- spatial hash build (src/sim/hash.cu:15-38, 106-133).
//
// The reference sorts (key, slot) pairs with CUB over all 32 key bits and
// clears two dense O(buckets) tables every tick. Here:
//   * keys use the reference's FP64 bucket arithmetic exactly (FP32 estimate,
//     FP64 only within the estimate's error of a bucket boundary);
//   * a stable LSD radix sort runs over only ceil(log2(buckets + 1)) bits;
//   * the dense {start, end} table is cleared only at the buckets the previous
//     build wrote (read from its sorted keys before they are overwritten);
//   * the ranges pass also writes a sorted-order 16-byte snapshot per cell --
//     position as FP32 offsets from its bucket's corner plus the packed bucket
//     coordinates -- so a neighbour separation is (bucket delta) * cell +
//     (offset delta) in FP32, streamed from contiguous records instead of three
//     FP64 arrays gathered through an index.
// Sorted output is the same as the reference's: stable order by key with
// ascending slots inside a bucket.
#include <cuda_runtime.h>

#include "kernels.h"

namespace agb {

namespace {

constexpr int RT = 256;           // radix threads per tile = keys per tile

__global__ void clear_prev_ranges_kernel(DevState* S, HashDev h) {
    const int32_t n = S->hash_count;
    AGB_FOR_CELLS(k, n) {
        const uint32_t key = h.keys_sorted[k];
        if (key < (uint32_t)h.buckets) h.ranges[key] = make_int2(0, 0);
    }
}

// key_kernel, src/sim/hash.cu:15-25
__global__ void key_kernel(DevState* S, HashDev h) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS(i, n) {
        h.vals[i] = (uint32_t)i;
        uint32_t key = (uint32_t)h.buckets;
        if (v.flags[i] & AGB_FLAG_OCCUPIED) {
            int32_t gx, gy, gz;
            hash_coords(h, v.x[i], v.y[i], v.z[i], gx, gy, gz);
            key = (uint32_t)((gz * h.ny + gy) * h.nx + gx);
        }
        h.keys[i] = key;
    }
}

// Per-tile digit histogram, digit-major: hist[d * tiles + t].
__global__ void __launch_bounds__(RT) radix_upsweep(DevState* S, const uint32_t* __restrict__ kin,
                                                   uint32_t* hist, int shift, int num_tiles) {
    __shared__ uint32_t cnt[256];
    const int tile = blockIdx.x;
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t e = (int64_t)tile * RT + threadIdx.x;
    if (e < S->count) atomicAdd(&cnt[(kin[e] >> shift) & 255u], 1u);
    __syncthreads();
    hist[threadIdx.x * num_tiles + tile] = cnt[threadIdx.x];
}

// Exclusive scan of each digit's row across tiles (one block per digit);
// totals[d] = the digit's count over all tiles.
__global__ void __launch_bounds__(1024) radix_scan_digits(uint32_t* hist, uint32_t* totals, int num_tiles) {
    __shared__ uint32_t part[1024];
    uint32_t* row = hist + (int64_t)blockIdx.x * num_tiles;
    const int t = threadIdx.x;
    const int per = (num_tiles + 1023) / 1024;
    const int b = t * per, e = b + per < num_tiles ? b + per : num_tiles;
    uint32_t s = 0;
    for (int i = b; i < e; ++i) s += row[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t > 0 ? part[t - 1] : 0u;
    for (int i = b; i < e; ++i) {
        const uint32_t x = row[i];
        row[i] = run;
        run += x;
    }
    if (t == 1023) totals[blockIdx.x] = part[1023];
}

// Stable scatter of one 256-key tile: rank = earlier same-digit keys in the
// warp (match_any) + same-digit keys in earlier warps of the tile; the global
// offset = (keys of smaller digits) + (same digit in earlier tiles).
__global__ void __launch_bounds__(RT) radix_downsweep(DevState* S, const uint32_t* __restrict__ kin,
                                                     const uint32_t* __restrict__ vin, uint32_t* kout,
                                                     uint32_t* vout, const uint32_t* __restrict__ offs,
                                                     const uint32_t* __restrict__ totals, int shift,
                                                     int num_tiles) {
    __shared__ uint32_t dbase[256];
    __shared__ uint32_t wcnt[RT / 32][256];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int tile = blockIdx.x;
    const int32_t n = S->count;
    const int64_t e = (int64_t)tile * RT + t;
    if ((int64_t)tile * RT >= n) return;                 // whole block beyond the live count
    // Exclusive scan of the 256 digit totals (every block recomputes it).
    dbase[t] = totals[t];
    for (int q = 0; q < RT / 32; ++q) wcnt[q][t] = 0;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const uint32_t v = t >= off ? dbase[t - off] : 0u;
        __syncthreads();
        dbase[t] += v;
        __syncthreads();
    }
    const uint32_t mybase = (t > 0 ? dbase[t - 1] : 0u);
    __syncthreads();
    dbase[t] = mybase + offs[t * num_tiles + tile];
    const bool valid = e < n;
    const uint32_t key = valid ? kin[e] : 0u;
    const uint32_t d = (key >> shift) & 255u;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, valid ? d : (0x100u | (unsigned)lane));
    if (valid && (peers & lt) == 0u) wcnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
        uint32_t pos = __popc(peers & lt);
        for (int q = 0; q < w; ++q) pos += wcnt[q][d];
        const uint32_t o = dbase[d] + pos;
        kout[o] = key;
        vout[o] = vin[e];
    }
}

// range_kernel (src/sim/hash.cu:29-38) + the sorted snapshot.
__global__ void ranges_kernel(DevState* S, HashDev h) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    if (blockIdx.x == 0 && threadIdx.x == 0) S->hash_count = n;
    AGB_FOR_CELLS(k, n) {
        const uint32_t key = h.keys_sorted[k];
        const uint32_t slot = h.vals_sorted[k];
        if (key < (uint32_t)h.buckets) {
            if (k == 0 || h.keys_sorted[k - 1] != key) h.ranges[key].x = k;
            if (k == n - 1 || h.keys_sorted[k + 1] != key) h.ranges[key].y = k + 1;
        }
        // Offsets from the bucket's corner, formed exactly in fixed point and
        // rounded once to FP32, plus the bucket coordinates (x, y: 11 bits; z: 10).
        int32_t gx, gy, gz;
        const double px = v.x[slot], py = v.y[slot], pz = v.z[slot];
        hash_coords(h, px, py, pz, gx, gy, gz);
        const float ox = __ll2float_rn(to_fix64(px, h.fix_k) - (h.org_fix[0] + gx * h.cell_fix)) * h.fix_inv_f;
        const float oy = __ll2float_rn(to_fix64(py, h.fix_k) - (h.org_fix[1] + gy * h.cell_fix)) * h.fix_inv_f;
        const float oz = __ll2float_rn(to_fix64(pz, h.fix_k) - (h.org_fix[2] + gz * h.cell_fix)) * h.fix_inv_f;
        h.rec[k] = make_float4(ox, oy, oz, __uint_as_float((uint32_t)gx | ((uint32_t)gy << 11) | ((uint32_t)gz << 22)));
    }
}

}  // namespace

void hash_build(DevState* S, const HashDev& h, int32_t capacity, uint32_t* kalt, uint32_t* valt,
                uint32_t* hist, int32_t grid_blocks, cudaStream_t s) {
    clear_prev_ranges_kernel<<<grid_blocks, 256, 0, s>>>(S, h);
    key_kernel<<<grid_blocks, 256, 0, s>>>(S, h);
    int bits = 0;
    while (bits < 32 && ((uint64_t)(uint32_t)h.buckets >> bits) != 0) ++bits;
    const int passes = (bits + 7) / 8;
    const int num_tiles = (capacity + RT - 1) / RT;
    uint32_t* totals = hist + (size_t)256 * num_tiles;
    uint32_t* kin = h.keys;
    uint32_t* vin = h.vals;
    for (int p = 0; p < passes; ++p) {
        uint32_t* kout = (p == passes - 1) ? h.keys_sorted : ((p & 1) ? h.keys : kalt);
        uint32_t* vout = (p == passes - 1) ? h.vals_sorted : ((p & 1) ? h.vals : valt);
        radix_upsweep<<<num_tiles, RT, 0, s>>>(S, kin, hist, p * 8, num_tiles);
        radix_scan_digits<<<256, 1024, 0, s>>>(hist, totals, num_tiles);
        radix_downsweep<<<num_tiles, RT, 0, s>>>(S, kin, vin, kout, vout, hist, totals, p * 8, num_tiles);
        kin = kout;
        vin = vout;
    }
    ranges_kernel<<<grid_blocks, 256, 0, s>>>(S, h);
}

}  // namespace agb
