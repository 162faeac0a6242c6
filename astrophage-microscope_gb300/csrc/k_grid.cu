// k_grid.cu -- FTCS conduction/diffusion and the fixed-point flush.
//
// HBM-bound: a pass reads each voxel once and writes it once (8 B per
// voxel-step). The 3-D kernel marches each thread up a z column keeping the
// below/centre/above values in registers, so every plane is fetched once from
// DRAM; in-plane neighbours come from L1. Arithmetic follows
// src/fields/diffuse.cu:19-44 operation for operation (explicitly rounded, no
// contraction), so nz == 1 reproduces the reference bit for bit.
#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.h"

namespace agb {

namespace {

__global__ void fill_kernel(float* v, int64_t n, float value) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = value;
}

struct Faces {
    int32_t bc[6];
    float val[6];
    float robin;
};

// diffuse_kernel's ghost (src/fields/diffuse.cu:27-36), per face.
__device__ __forceinline__ float ghost(const Faces& f, int face, float c) {
    if (f.bc[face] == AGB_BC_DIRICHLET) return f.val[face];
    if (f.bc[face] == AGB_BC_ROBIN) return fs(c, fm(f.robin, fs(c, f.val[face])));
    return c;
}

// 2-D (nz == 1): the reference's 5-point formula.
__global__ void __launch_bounds__(256) ftcs2d_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                     int32_t nx, int32_t ny, float coeff, Faces f) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    const int64_t idx = (int64_t)j * nx + i;
    const float c = src[idx];
    const float l = (i > 0) ? src[idx - 1] : ghost(f, AGB_FACE_XMIN, c);
    const float r = (i < nx - 1) ? src[idx + 1] : ghost(f, AGB_FACE_XMAX, c);
    const float d = (j > 0) ? src[idx - nx] : ghost(f, AGB_FACE_YMIN, c);
    const float u = (j < ny - 1) ? src[idx + nx] : ghost(f, AGB_FACE_YMAX, c);
    // c + coeff * (l + r + d + u - 4.0f * c)
    const float sum = fs(fa(fa(fa(l, r), d), u), fm(4.0f, c));
    dst[idx] = fa(c, fm(coeff, sum));
}

// 3-D 7-point: c + coeff * (l + r + d + u + b + t - 6c), each thread marching
// ZCHUNK planes of one (i, j) column.
constexpr int ZCHUNK = 8;

__global__ void __launch_bounds__(256) ftcs3d_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                     int32_t nx, int32_t ny, int32_t nz, float coeff,
                                                     Faces f) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t j = blockIdx.y * blockDim.y + threadIdx.y;
    const int32_t k0 = blockIdx.z * ZCHUNK;
    if (i >= nx || j >= ny) return;
    const int64_t plane = (int64_t)nx * ny;
    const int64_t col = (int64_t)j * nx + i;
    int32_t k1 = k0 + ZCHUNK;
    if (k1 > nz) k1 = nz;
    float c = __ldg(src + col + plane * k0);
    float below = (k0 > 0) ? __ldg(src + col + plane * (k0 - 1)) : ghost(f, AGB_FACE_ZMIN, c);
#pragma unroll 4
    for (int32_t k = k0; k < k1; ++k) {
        const int64_t idx = col + plane * k;
        const float above = (k < nz - 1) ? __ldg(src + idx + plane) : ghost(f, AGB_FACE_ZMAX, c);
        const float l = (i > 0) ? __ldg(src + idx - 1) : ghost(f, AGB_FACE_XMIN, c);
        const float r = (i < nx - 1) ? __ldg(src + idx + 1) : ghost(f, AGB_FACE_XMAX, c);
        const float d = (j > 0) ? __ldg(src + idx - nx) : ghost(f, AGB_FACE_YMIN, c);
        const float u = (j < ny - 1) ? __ldg(src + idx + nx) : ghost(f, AGB_FACE_YMAX, c);
        const float b = (k > 0) ? below : ghost(f, AGB_FACE_ZMIN, c);
        const float sum = fs(fa(fa(fa(fa(fa(l, r), d), u), b), above), fm(6.0f, c));
        dst[idx] = fa(c, fm(coeff, sum));
        below = c;
        c = above;
    }
}


// ---------------------------------------------------------------------------
// 3-D FTCS with TMA-staged planes. A CTA owns a TX x TY (x, y) tile and
// marches ZC planes of z. Input planes (tile plus a one-voxel halo) arrive by
// cp.async.bulk.tensor into a ring of NBUF shared-memory buffers, each guarded
// by an mbarrier; the plane three ahead is in flight while one is computed, so
// every voxel is fetched once per pass and read from shared memory six more
// times. The x halo starts four elements early because a tiled TMA copy must
// begin on a 16-byte boundary; out-of-range coordinates (negative or past the
// grid) are zero-filled by the copy and never used -- boundary voxels take the
// ghost values exactly as the plain kernel does. Same arithmetic, same order,
// so the two kernels agree bit for bit.
// ---------------------------------------------------------------------------
constexpr int TX = 64, TY = 16, HX = 4;                 // HX: leading x halo (alignment)
constexpr int BXW = TX + 2 * HX, BYH = TY + 2;          // box 72 x 18
constexpr int PLANE_BYTES = BXW * BYH * 4;              // 5184
constexpr int PLANE_STRIDE = (PLANE_BYTES + 127) / 128 * 128;
constexpr int NBUF = 4;
constexpr uint32_t WAIT_LIMIT = 1u << 26;               // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after WAIT_LIMIT polls and reports it.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err) {
    for (uint32_t it = 0; it < WAIT_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicCAS(err, 0u, 4u);    // ERR_TMA_TIMEOUT
    return false;
}
__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, uint64_t* bar, int x, int y,
                                               int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__global__ void __launch_bounds__(256) ftcs3d_tma_kernel(const __grid_constant__ CUtensorMap src_map,
                                                         float* __restrict__ dst, int32_t nx, int32_t ny,
                                                         int32_t nz, int32_t zc, float coeff, Faces f,
                                                         uint32_t* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + NBUF * PLANE_STRIDE);
    const int tid = threadIdx.x;
    const int32_t x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, k0 = blockIdx.z * zc;
    const int32_t k1 = k0 + zc < nz ? k0 + zc : nz;
    const int nplanes = (k1 - k0) + 2;                  // z = k0-1 .. k1
    auto buf = [&](int q) { return reinterpret_cast<float*>(smem + (q % NBUF) * PLANE_STRIDE); };
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(&bar[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        for (int q = 0; q < NBUF && q < nplanes; ++q) {
            mbar_expect_tx(&bar[q % NBUF], PLANE_BYTES);
            tma_load_plane(buf(q), &src_map, &bar[q % NBUF], x0 - HX, y0 - 1, k0 - 1 + q);
        }
    }
    const int tx = tid & (TX - 1), ty0 = tid >> 6;       // 4 output rows per thread
    const int32_t i = x0 + tx;
    // Every wait is bounded, and the go/stop decision after it is made
    // block-wide (__syncthreads_and), so a timeout can never leave part of the
    // block waiting at a barrier the rest has abandoned.
    bool ok = true;
    for (int q = 0; q < 3; ++q) ok = mbar_wait(&bar[q % NBUF], (uint32_t)((q / NBUF) & 1), err) && ok;
    ok = __syncthreads_and(ok);
    for (int32_t k = k0; k < k1 && ok; ++k) {
        const int q = k - k0 + 1;                       // plane index of z = k
        if (k > k0) {
            ok = mbar_wait(&bar[(q + 1) % NBUF], (uint32_t)(((q + 1) / NBUF) & 1), err);
            ok = __syncthreads_and(ok);
            if (!ok) break;
        }
        const float* pb = buf(q - 1);
        const float* pc = buf(q);
        const float* pa = buf(q + 1);
        if (i < nx) {
#pragma unroll
            for (int r = 0; r < TY / 4; ++r) {
                const int ty = ty0 + 4 * r;
                const int32_t j = y0 + ty;
                if (j >= ny) continue;
                const int s = (ty + 1) * BXW + (tx + HX);
                const float c = pc[s];
                const float l = (i > 0) ? pc[s - 1] : ghost(f, AGB_FACE_XMIN, c);
                const float rr = (i < nx - 1) ? pc[s + 1] : ghost(f, AGB_FACE_XMAX, c);
                const float d = (j > 0) ? pc[s - BXW] : ghost(f, AGB_FACE_YMIN, c);
                const float u = (j < ny - 1) ? pc[s + BXW] : ghost(f, AGB_FACE_YMAX, c);
                const float b = (k > 0) ? pb[s] : ghost(f, AGB_FACE_ZMIN, c);
                const float a = (k < nz - 1) ? pa[s] : ghost(f, AGB_FACE_ZMAX, c);
                const float sum = fs(fa(fa(fa(fa(fa(l, rr), d), u), b), a), fm(6.0f, c));
                dst[(int64_t)k * nx * ny + (int64_t)j * nx + i] = fa(c, fm(coeff, sum));
            }
        }
        __syncthreads();                                // everyone is done with plane q-1
        if (tid == 0 && q - 1 + NBUF < nplanes) {
            const int qn = q - 1 + NBUF;
            mbar_expect_tx(&bar[qn % NBUF], PLANE_BYTES);
            tma_load_plane(buf(qn), &src_map, &bar[qn % NBUF], x0 - HX, y0 - 1, k0 - 1 + qn);
        }
    }
    // A CTA that gave up waits (bounded) for its own copies before leaving, so
    // no transfer lands in shared memory after the block has exited.
    if (!ok && tid == 0) {
        for (int q = 0; q < nplanes && q < NBUF; ++q) {
            for (uint32_t it = 0; it < WAIT_LIMIT; ++it)
                if (mbar_try_wait(&bar[q], 0) || mbar_try_wait(&bar[q], 1)) break;
        }
    }
}

// Sparse flush: every occupied cell exchanges its voxel's accumulator for zero;
// exactly one thread per voxel sees the nonzero sum and folds it in, so the
// result equals the reference's dense flush over all voxels (a voxel without a
// depositing cell holds zero). Optionally also zeroes a per-voxel demand
// accumulator of the same grid (the CO2 rationing buffer).
__global__ void flush_by_cells_kernel(DevState* S, GridDev g, unsigned long long* demand) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS(i, n) {
        if (!(v.flags[i] & AGB_FLAG_OCCUPIED)) continue;
        const int64_t idx = grid_nearest(g, (float)v.x[i], (float)v.y[i], (float)v.z[i]);
        const unsigned long long raw = atomicExch(&g.deposit[idx], 0ull);
        if (raw != 0ull) {
            // (float)(raw / scale): FP32 scaling; identical to the reference's
            // double division except in the last bit of a ~1e-2 increment.
            g.value[idx] = fa(g.value[idx], (float)(long long)raw * g.inv_scale_f);
        }
        if (demand) demand[idx] = 0ull;
    }
}

}  // namespace

void launch_fill(float* v, int64_t n, float value, cudaStream_t s) {
    const int64_t blocks = (n + 255) / 256;
    fill_kernel<<<(unsigned)(blocks > 4096 ? 4096 : blocks), 256, 0, s>>>(v, n, value);
}

void launch_ftcs(const GridDev& g, const float* src, float* dst, float coeff, const int32_t* bc,
                 const float* face, float robin, const CUtensorMap* src_map, uint32_t* err, cudaStream_t s) {
    Faces f;
    for (int k = 0; k < 6; ++k) { f.bc[k] = bc[k]; f.val[k] = face[k]; }
    f.robin = robin;
    if (g.nz > 1 && src_map != nullptr) {
        // z planes per CTA: as many as keep the grid at >= 4 CTAs per SM (fewer
        // planes per CTA re-read more halo planes, which come from L2), 2..16.
        static int sms = 0;
        if (sms == 0) { int d = 0; cudaGetDevice(&d); cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d); }
        const int64_t tiles = (int64_t)((g.nx + TX - 1) / TX) * ((g.ny + TY - 1) / TY);
        int32_t zc = (int32_t)(g.nz * tiles / (4 * (int64_t)(sms > 0 ? sms : 148)));
        zc = zc < 2 ? 2 : (zc > 16 ? 16 : zc);
        const dim3 grid((g.nx + TX - 1) / TX, (g.ny + TY - 1) / TY, (g.nz + zc - 1) / zc);
        ftcs3d_tma_kernel<<<grid, 256, NBUF * PLANE_STRIDE + 64, s>>>(*src_map, dst, g.nx, g.ny, g.nz, zc, coeff, f,
                                                                      err);
        return;
    }
    if (g.nz == 1) {
        const dim3 block(32, 8);
        const dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8);
        ftcs2d_kernel<<<grid, block, 0, s>>>(src, dst, g.nx, g.ny, coeff, f);
    } else {
        const dim3 block(32, 8);
        const dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + ZCHUNK - 1) / ZCHUNK);
        ftcs3d_kernel<<<grid, block, 0, s>>>(src, dst, g.nx, g.ny, g.nz, coeff, f);
    }
}

void launch_flush_by_cells(DevState* S, GridDev g, unsigned long long* demand, int32_t grid_blocks,
                           cudaStream_t s) {
    flush_by_cells_kernel<<<grid_blocks, 256, 0, s>>>(S, g, demand);
}

}  // namespace agb

namespace agb {

// A 3-D tensor map over one field buffer for ftcs3d_tma_kernel: box 72 x 18 x 1
// floats. Returns false (plain kernel used instead) when the driver entry
// point is unavailable or the grid's row pitch is not a multiple of 16 bytes.
bool make_plane_map(CUtensorMap* map, float* base, int32_t nx, int32_t ny, int32_t nz) {
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return false;
        encode = reinterpret_cast<Encode>(fn);
    }
    if (nz <= 1 || (nx * 4) % 16 != 0) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)BXW, (cuuint32_t)BYH, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace agb
