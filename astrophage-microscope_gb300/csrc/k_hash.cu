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

#include "cells.h"
#include "kernels.h"

namespace agb {

namespace {

// ---------------------------------------------------------------------------
// Stable LSD radix sort, one kernel per 8-bit pass (a single-sweep scheme):
//   * key_hist_kernel (below) writes every key once and counts the digits of
//     all passes (global histograms, then their exclusive scans in each pass);
//   * radix_pass_kernel: a CTA takes the next 1024- or 2048-key tile (tile order = the
//     order CTAs start, so every tile it waits on is already running), ranks
//     its keys stably (warp match_any per 32-key group, then a per-digit scan
//     over the tile's 64 groups), publishes its per-digit count, looks back
//     over earlier tiles' published counts/prefixes (decoupled look-back) and
//     scatters. Look-back waits are bounded; a timeout sets the error word and
//     the CTA writes nothing.
// ---------------------------------------------------------------------------
constexpr int SORT_THREADS = 256;
// Digit histograms of all passes: [4][256] for 8-bit digits or [3][512] for 9-bit.
constexpr int HIST_WORDS = 1536;
constexpr uint32_t FLAG_AGG = 1u << 30, FLAG_PRE = 2u << 30, VALUE_MASK = (1u << 30) - 1u;
constexpr int LOOKBACK_BATCH = 8;                                // predecessor words read per round trip
constexpr uint32_t LOOKBACK_LIMIT = 1u << 24;

// PER keys per thread: a tile is 256 * PER keys in 8 * PER warp-groups; RB
// bits per digit (8 or 9: 256 or 512 digits, DPT digits per thread).
template <int PER, int RB>
__device__ __forceinline__ void radix_pass_kernel_body(DevState* S, const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                                                       uint32_t* __restrict__ vout,
                                                       const uint32_t* __restrict__ ghist, uint32_t* status,
                                                       uint32_t* tile_counter, int shift, Blk blk) {
    constexpr int NB = 1 << RB;
    constexpr int DPT = NB / SORT_THREADS;
    constexpr int SORT_TILE = SORT_THREADS * PER;
    constexpr int SORT_GROUPS = SORT_TILE / 32;
    __shared__ uint16_t cnt[SORT_GROUPS][NB];      // per group and digit: count, then exclusive prefix
    __shared__ uint32_t dbase[NB];                 // global base of each digit for this tile
    __shared__ uint32_t part[SORT_THREADS];
    __shared__ uint32_t tile_id;
    __shared__ int ok_all;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int32_t n = S->count;
    const int ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    if (t == 0) tile_id = atomicAdd(tile_counter, 1u);
    for (int g = 0; g < SORT_GROUPS; ++g)
#pragma unroll
        for (int q = 0; q < DPT; ++q) cnt[g][t + q * SORT_THREADS] = 0;
    __syncthreads();
    const int tile = (int)tile_id;
    if (tile >= ntiles) return;                      // block-uniform
    const int64_t base = (int64_t)tile * SORT_TILE;
    // Element order inside the tile: e = k * 256 + t; group = k * 8 + w.
    uint32_t key[PER], dig[PER], rank[PER];
    unsigned peers_lt[PER];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int64_t e = base + k * SORT_THREADS + t;
        const bool valid = e < n;
        key[k] = valid ? kin[e] : 0xFFFFFFFFu;
        dig[k] = valid ? (key[k] >> shift) & (uint32_t)(NB - 1) : (uint32_t)NB + (unsigned)lane;   // invalid: unique
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, dig[k]);
        peers_lt[k] = __popc(peers & lt);
        if (valid && (peers & lt) == 0u) cnt[k * 8 + w][dig[k]] = (uint16_t)__popc(peers);
    }
    __syncthreads();
    // Exclusive scan of each digit's column over the groups (thread t owns
    // digits t, t + 256, ...).
    uint32_t my_count[DPT];
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        const int d = t + q * SORT_THREADS;
        uint32_t run = 0;
        for (int g = 0; g < SORT_GROUPS; ++g) {
            const uint32_t c = cnt[g][d];
            cnt[g][d] = (uint16_t)run;
            run += c;
        }
        my_count[q] = run;                           // keys of digit d in this tile
    }
    // Publish the aggregates (tile 0 publishes its inclusive prefixes
    // directly), then look back for the exclusive prefixes over earlier tiles.
    uint32_t* st = status + (int64_t)tile * NB;
#pragma unroll
    for (int q = 0; q < DPT; ++q)
        atomicExch(&st[t + q * SORT_THREADS], (tile == 0 ? FLAG_PRE : FLAG_AGG) | my_count[q]);
    // Look back in batches: the words of up to LOOKBACK_BATCH predecessors are
    // loaded together (one round trip), nearest first; summing stops at the
    // nearest inclusive prefix. A word not yet published is polled again.
    uint32_t excl[DPT];
    bool ok = true;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        const int d = t + q * SORT_THREADS;
        excl[q] = 0;
        for (int j0 = tile - 1; j0 >= 0 && ok;) {
            const int nb = j0 + 1 < LOOKBACK_BATCH ? j0 + 1 : LOOKBACK_BATCH;
            uint32_t v[LOOKBACK_BATCH];
#pragma unroll
            for (int r = 0; r < LOOKBACK_BATCH; ++r)
                v[r] = r < nb ? *(volatile const uint32_t*)(status + (int64_t)(j0 - r) * NB + d) : FLAG_PRE;
            bool done = false;
            for (int r = 0; r < nb && ok && !done; ++r) {
                uint32_t it = 0;
                while (!(v[r] & (FLAG_AGG | FLAG_PRE)) && it < LOOKBACK_LIMIT) {
                    v[r] = *(volatile const uint32_t*)(status + (int64_t)(j0 - r) * NB + d);
                    ++it;
                }
                if (!(v[r] & (FLAG_AGG | FLAG_PRE))) { ok = false; set_error(S, 5u); break; }
                excl[q] += v[r] & VALUE_MASK;
                if (v[r] & FLAG_PRE) done = true;
            }
            if (done) break;
            j0 -= nb;
        }
    }
    if (tile > 0 && ok) {
        __threadfence();
#pragma unroll
        for (int q = 0; q < DPT; ++q) atomicExch(&st[t + q * SORT_THREADS], FLAG_PRE | (excl[q] + my_count[q]));
    }
    // Digit base = (keys of smaller digits over all tiles) + (this digit in
    // earlier tiles): an exclusive scan of the global histogram, thread t
    // holding digits t * DPT .. t * DPT + DPT - 1.
    uint32_t hv[DPT], loc = 0;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        hv[q] = ghist[t * DPT + q];
        loc += hv[q];
    }
    part[t] = loc;
    if (t == 0) ok_all = 1;
    __syncthreads();
    if (!ok) ok_all = 0;
    for (int off = 1; off < SORT_THREADS; off <<= 1) {
        const uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t acc = t > 0 ? part[t - 1] : 0u;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        dbase[t * DPT + q] = acc;
        acc += hv[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < DPT; ++q) dbase[t + q * SORT_THREADS] += excl[q];
    __syncthreads();
    if (!ok_all) return;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int64_t e = base + k * SORT_THREADS + t;
        if (e >= n) continue;
        const uint32_t d = dig[k];
        rank[k] = dbase[d] + cnt[k * 8 + w][d] + peers_lt[k];
        kout[rank[k]] = key[k];
        vout[rank[k]] = vin[e];
    }
}

template <int PER, int RB>
__global__ void __launch_bounds__(SORT_THREADS) radix_pass_kernel(DevState* S, const uint32_t* __restrict__ kin,
                                                                  const uint32_t* __restrict__ vin,
                                                                  uint32_t* __restrict__ kout,
                                                                  uint32_t* __restrict__ vout,
                                                                  const uint32_t* __restrict__ ghist,
                                                                  uint32_t* status, uint32_t* tile_counter,
                                                                  int shift) {
    pdl_wait();
    radix_pass_kernel_body<PER, RB>(S, kin, vin, kout, vout, ghist, status, tile_counter, shift, grid_blk());
}

// The hash build's first pass, fused: clear the bucket ranges the previous
// build wrote, compute every slot's key (key_kernel, src/sim/hash.cu:15-25)
// and count the digits of all radix passes.
__device__ __forceinline__ void key_hist_kernel_body(DevState* S, const HashDev& h, uint32_t* __restrict__ ghist,
                                                     int passes, int rb, Blk blk) {
    __shared__ uint32_t hs[HIST_WORDS];              // [pass][digit], 1 << rb digits per pass
    const uint32_t nbins = 1u << rb;
    for (int i = threadIdx.x; i < HIST_WORDS; i += blockDim.x) hs[i] = 0u;
    __syncthreads();
    const SoA v = S->cur;
    const int32_t n = S->count, nprev = S->hash_count;
    const int32_t m = n > nprev ? n : nprev;
    for (int64_t i = blk.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)blk.n * blockDim.x) {
        if (i < nprev) {
            const uint32_t old = h.keys_sorted[i];
            if (old < (uint32_t)h.buckets) {
                h.ranges[old] = make_int2(0, 0);
                if (i == 0 || h.keys_sorted[i - 1] != old) atomicAnd(&h.occ[old >> 5], ~(1u << (old & 31u)));
            }
        }
        if (i < n) {
            h.vals[i] = (uint32_t)i;
            uint32_t key = (uint32_t)h.buckets;
            if (v.flags[i] & AGB_FLAG_OCCUPIED) {
                int32_t gx, gy, gz;
                hash_coords(h, v.x[i], v.y[i], v.z[i], gx, gy, gz);
                key = (uint32_t)((gz * h.ny + gy) * h.nx + gx);
            }
            h.keys[i] = key;
            for (int p = 0; p < passes; ++p) atomicAdd(&hs[p * nbins + ((key >> (rb * p)) & (nbins - 1u))], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * (int)nbins; i += blockDim.x) {
        const uint32_t c = hs[i];
        if (c) atomicAdd(&ghist[i], c);
    }
}

__global__ void __launch_bounds__(256) key_hist_kernel(DevState* S, HashDev h, uint32_t* __restrict__ ghist,
                                                       int passes, int rb) {
    pdl_wait();
    key_hist_kernel_body(S, h, ghist, passes, rb, grid_blk());
}

// range_kernel (src/sim/hash.cu:29-38) + the sorted snapshot.
__device__ __forceinline__ void ranges_kernel_body(DevState* S, const HashDev& h, Blk blk) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    if (blk.x == 0 && threadIdx.x == 0) S->hash_count = n;
    AGB_FOR_CELLS_B(k, blk, n) {
        const uint32_t key = h.keys_sorted[k];
        const uint32_t slot = h.vals_sorted[k];
        if (key < (uint32_t)h.buckets) {
            if (k == 0 || h.keys_sorted[k - 1] != key) {
                h.ranges[key].x = k;
                atomicOr(&h.occ[key >> 5], 1u << (key & 31u));
            }
            if (k == n - 1 || h.keys_sorted[k + 1] != key) h.ranges[key].y = k + 1;
        }
        // Offsets from the bucket's corner, formed exactly in fixed point and
        // rounded once to FP32, plus the bucket coordinates (x, y: 11 bits; z: 10).
        int32_t gx, gy, gz;
        const double px = v.x[slot], py = v.y[slot], pz = v.z[slot];
        hash_coords(h, px, py, pz, gx, gy, gz);
        const float ox = ll_to_f(to_fix64(px, h.fix_k) - (h.org_fix[0] + gx * h.cell_fix)) * h.fix_inv_f;
        const float oy = ll_to_f(to_fix64(py, h.fix_k) - (h.org_fix[1] + gy * h.cell_fix)) * h.fix_inv_f;
        const float oz = ll_to_f(to_fix64(pz, h.fix_k) - (h.org_fix[2] + gz * h.cell_fix)) * h.fix_inv_f;
        h.rec[k] = make_float4(ox, oy, oz, __uint_as_float((uint32_t)gx | ((uint32_t)gy << 11) | ((uint32_t)gz << 22)));
    }
}

__global__ void ranges_kernel(DevState* S, HashDev h) {
    pdl_wait();
    ranges_kernel_body(S, h, grid_blk());
}

// Batched hash builds (agb_batch). A chamber's sort scratch is laid out as in
// hash_build: [HIST_WORDS] digit histograms | [4] tile counters | per pass
// [max_tiles][1 << rb] look-back words; pass p reads the keys pass p - 1 wrote.
__device__ __forceinline__ uint32_t hash_scratch_words(const ChamberArgs& a) {
    return (uint32_t)HIST_WORDS + 4u + (uint32_t)a.passes * (uint32_t)a.max_tiles * (1u << a.radix_bits);
}
AGB_BATCHED(hash_clear_batch, 256, {
    const uint32_t words = hash_scratch_words(a);
    for (uint32_t i = (uint32_t)blk.x * blockDim.x + threadIdx.x; i < words; i += (uint32_t)blk.n * blockDim.x)
        a.hist[i] = 0u;
})
AGB_BATCHED(key_hist_batch, 256, key_hist_kernel_body(a.S, a.c.h, a.hist, a.passes, a.radix_bits, blk))
AGB_BATCHED(ranges_batch, 256, ranges_kernel_body(a.S, a.c.h, blk))

template <int PER, int RB>
__global__ void __launch_bounds__(SORT_THREADS) radix_batch(const ChamberArgs* __restrict__ tab,
                                                            const uint32_t* __restrict__ map, int32_t pass) {
    pdl_wait();
    int32_t ch, x;
    batch_block(map, ch, x);
    const ChamberArgs& a = tab[ch];
    const HashDev& h = a.c.h;
    const bool odd_in = ((pass - 1) & 1) != 0;
    const uint32_t* kin = pass == 0 ? h.keys : (odd_in ? h.keys : a.kalt);
    const uint32_t* vin = pass == 0 ? h.vals : (odd_in ? h.vals : a.valt);
    uint32_t* kout = pass == a.passes - 1 ? h.keys_sorted : ((pass & 1) ? h.keys : a.kalt);
    uint32_t* vout = pass == a.passes - 1 ? h.vals_sorted : ((pass & 1) ? h.vals : a.valt);
    uint32_t* counters = a.hist + HIST_WORDS;
    uint32_t* status = counters + 4 + (size_t)pass * a.max_tiles * (1 << RB);
    radix_pass_kernel_body<PER, RB>(a.S, kin, vin, kout, vout, a.hist + pass * (1 << RB), status, counters + pass,
                                    pass * RB, Blk{x, a.nblk});
}

}  // namespace

// Sort shape for a world: digit passes and width (9-bit digits when that
// saves a pass and tiles are 1024 keys, whose counts then still fit static
// shared memory), tiles per pass and tile size (1024 keys up to 256k cells).
void hash_sort_shape(const HashDev& h, int32_t capacity, int32_t& passes, int32_t& max_tiles, bool& per4,
                     int32_t& radix_bits) {
    int bits = 0;
    while (bits < 32 && ((uint64_t)(uint32_t)h.buckets >> bits) != 0) ++bits;
    per4 = capacity <= (256 << 10);
    const int p8 = (bits + 7) / 8, p9 = (bits + 8) / 9;
    radix_bits = (per4 && p9 < p8 && p9 * 512 <= HIST_WORDS) ? 9 : 8;
    passes = radix_bits == 9 ? p9 : p8;
    const int tile_keys = SORT_THREADS * (per4 ? 4 : 8);
    max_tiles = (capacity + tile_keys - 1) / tile_keys;
}

int32_t hash_clear_blocks(int32_t passes, int32_t max_tiles, int32_t radix_bits) {
    const int64_t words = HIST_WORDS + 4 + (int64_t)passes * max_tiles * (1 << radix_bits);
    const int64_t b = (words + 4 * 256 - 1) / (4 * 256);
    return (int32_t)(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

bool launch_batched_hash(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                         cudaStream_t s) {
    const unsigned g = (unsigned)blocks;
    switch (st) {
        case BStage::HashClear: launch_k(hash_clear_batch, g, 256, 0, s, tab, map); return true;
        case BStage::KeyHist: launch_k(key_hist_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Radix4: launch_k(radix_batch<4, 8>, g, SORT_THREADS, 0, s, tab, map, arg); return true;
        case BStage::Radix4x9: launch_k(radix_batch<4, 9>, g, SORT_THREADS, 0, s, tab, map, arg); return true;
        case BStage::Radix8: launch_k(radix_batch<8, 8>, g, SORT_THREADS, 0, s, tab, map, arg); return true;
        case BStage::Ranges: launch_k(ranges_batch, g, 256, 0, s, tab, map); return true;
        default: return false;
    }
}

void hash_build(DevState* S, const HashDev& h, int32_t capacity, uint32_t* kalt, uint32_t* valt,
                uint32_t* hist, int32_t grid_blocks, cudaStream_t s) {
    int32_t passes = 0, max_tiles = 0, rb = 8;
    bool per4 = true;
    hash_sort_shape(h, capacity, passes, max_tiles, per4, rb);
    const int nb = 1 << rb;
    // hist layout: [HIST_WORDS] digit histograms | [4] tile counters | [passes][max_tiles][nb] status words.
    uint32_t* ghist = hist;
    uint32_t* counters = hist + HIST_WORDS;
    uint32_t* status = counters + 4;
    cudaMemsetAsync(hist, 0, sizeof(uint32_t) * (HIST_WORDS + 4 + (size_t)passes * max_tiles * nb), s);
    launch_k(key_hist_kernel, grid_blocks, 256, 0, s, S, h, ghist, passes, rb);
    uint32_t* kin = h.keys;
    uint32_t* vin = h.vals;
    for (int p = 0; p < passes; ++p) {
        uint32_t* kout = (p == passes - 1) ? h.keys_sorted : ((p & 1) ? h.keys : kalt);
        uint32_t* vout = (p == passes - 1) ? h.vals_sorted : ((p & 1) ? h.vals : valt);
        uint32_t* st = status + (size_t)p * max_tiles * nb;
        if (!per4)
            launch_k(radix_pass_kernel<8, 8>, max_tiles, SORT_THREADS, 0, s, S, kin, vin, kout, vout, ghist + p * nb,
                     st, counters + p, p * rb);
        else if (rb == 9)
            launch_k(radix_pass_kernel<4, 9>, max_tiles, SORT_THREADS, 0, s, S, kin, vin, kout, vout, ghist + p * nb,
                     st, counters + p, p * rb);
        else
            launch_k(radix_pass_kernel<4, 8>, max_tiles, SORT_THREADS, 0, s, S, kin, vin, kout, vout, ghist + p * nb,
                     st, counters + p, p * rb);
        kin = kout;
        vin = vout;
    }
    launch_k(ranges_kernel, grid_blocks, 256, 0, s, S, h);
}

// Enough for any sort shape at this capacity: 4 passes of 256 digits or 3 of
// 512 per tile.
size_t hash_sort_scratch_words(int32_t capacity) {
    const int per = capacity <= (256 << 10) ? 4 : 8;
    const size_t tile_keys = (size_t)SORT_THREADS * per;
    const size_t max_tiles = ((size_t)capacity + tile_keys - 1) / tile_keys;
    return HIST_WORDS + 4 + (size_t)HIST_WORDS * max_tiles;
}

}  // namespace agb
