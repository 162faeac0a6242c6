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

#include <cstdio>
#include <cstdlib>

#include "cells.h"
#include "kernels.h"

namespace agb {

namespace {

__global__ void fill_kernel(float* v, int64_t n, float value) {
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = value;
}

// brush_kernel (src/fields/diffuse.cu:62-77): value += amount * (1 - t^2)^2 with
// t = r / radius, r the in-plane distance of the voxel centre from (cx, cy),
// for r <= radius. The launch covers the disc's bounding box of columns
// [x0, x0 + bw) x [y0, y0 + bh) on every z plane (nz == 1 is the reference's
// grid; a 3-D grid takes the same disc on each plane). Explicitly rounded, in
// the reference's order of operations.
__global__ void brush_kernel(float* v, GridDev g, float cx, float cy, float radius, float amount,
                             int32_t x0, int32_t y0, int32_t bw, int32_t bh) {
    pdl_wait();
    const int64_t n = (int64_t)bw * bh * g.nz;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = x0 + (int32_t)(k % bw);
        const int64_t r2 = k / bw;
        const int32_t j = y0 + (int32_t)(r2 % bh);
        const int32_t z = (int32_t)(r2 / bh);
        const float x = fs(fm(fa((float)i, 0.5f), g.dxf), g.hx);
        const float y = fs(fm(fa((float)j, 0.5f), g.dxf), g.hy);
        const float ex = fs(x, cx), ey = fs(y, cy);
        const float r = sqrtf(fa(fm(ex, ex), fm(ey, ey)));
        if (r > radius) continue;
        const float t = __fdiv_rn(r, radius);
        const float q = fs(1.0f, fm(t, t));
        const int64_t idx = i + (int64_t)g.nx * (j + (int64_t)g.ny * z);
        v[idx] = fa(v[idx], fm(amount, fm(q, q)));
    }
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
    pdl_wait();
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
    pdl_wait();
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
// 3-D FTCS with TMA-staged planes. A CTA owns a (4*LX) x (256/LX*RPT) tile of
// (x, y) and marches zc planes of z. Input planes (tile plus a one-voxel halo)
// arrive by cp.async.bulk.tensor into a ring of NBUF shared-memory buffers,
// each guarded by an mbarrier. A thread owns four consecutive x voxels in RPT
// rows: the centre row comes in as one 16-byte shared load and the z
// neighbours live in registers (the thread marches up its columns), so four
// voxels cost five shared loads and one 16-byte global store. Boundary voxels
// take ghost values in registers; only warps on the grid's faces run that code.
// The x halo starts four elements early because a tiled TMA copy must begin on
// a 16-byte boundary; out-of-range coordinates (negative or past the grid) are
// zero-filled by the copy and never used. Same arithmetic, same order as the
// plain kernels, so every kernel here agrees bit for bit.
// ---------------------------------------------------------------------------
constexpr int HX = 4;                                   // x halo each side (alignment)
constexpr int NBUF = 4;                                 // ring: 2 planes in use, 2 in flight
constexpr uint32_t WAIT_LIMIT = 1u << 26;               // bounded mbarrier polls

template <int LX, int RPT>
struct TmaTile {
    static constexpr int TXW = 4 * LX;                  // voxels along x
    static constexpr int ROWS = 256 / LX;               // thread rows
    static constexpr int TYH = ROWS * RPT;              // voxels along y
    static constexpr int BXW = TXW + 2 * HX;            // box width (floats)
    static constexpr int BYH = TYH + 2;                 // box height
    static constexpr int PLANE_BYTES = BXW * BYH * 4;
    static constexpr int PLANE_STRIDE = (PLANE_BYTES + 127) / 128 * 128;
    static constexpr int SMEM = NBUF * PLANE_STRIDE + 64;
};

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
// Orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (TMA) accesses. Every thread that read a ring slot runs it
// before the barrier after which the slot is refilled: a barrier alone orders
// the generic proxy only, and a shared load still in flight when the barrier
// completes (its value not yet consumed) could otherwise return the refill.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, uint64_t* bar, int x, int y,
                                               int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float4 ghost4(const Faces& f, int face, float4 c) {
    return make_float4(ghost(f, face, c.x), ghost(f, face, c.y), ghost(f, face, c.z), ghost(f, face, c.w));
}
// c + coeff * (l + r + d + u + b + a - 6c), the plain kernels' order.
__device__ __forceinline__ float ftcs7(float c, float l, float r, float d, float u, float b, float a, float coeff) {
    const float sum = fs(fa(fa(fa(fa(fa(l, r), d), u), b), a), fm(6.0f, c));
    return fa(c, fm(coeff, sum));
}

// One CTA's tile (bx, by) and z chunk bz of a pass, reading the source through
// the tensor map at `src_map` (a kernel parameter or a table entry).
template <int LX, int RPT>
__device__ __forceinline__ void ftcs3d_tma_body(const CUtensorMap* src_map, float* __restrict__ dst, int32_t nx,
                                                int32_t ny, int32_t nz, int32_t zc, float coeff, const Faces& f,
                                                uint32_t* err, int32_t bx, int32_t by, int32_t bz) {
    using T = TmaTile<LX, RPT>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + NBUF * T::PLANE_STRIDE);
    const int tid = threadIdx.x;
    const int32_t x0 = bx * T::TXW, y0 = by * T::TYH, k0 = bz * zc;
    const int32_t k1 = k0 + zc < nz ? k0 + zc : nz;
    const int nplanes = (k1 - k0) + 2;                  // plane q holds z = k0 - 1 + q
    auto buf = [&](int q) { return reinterpret_cast<const float*>(smem + (q % NBUF) * T::PLANE_STRIDE); };
    auto issue = [&](int q) {
        mbar_expect_tx(&bar[q % NBUF], T::PLANE_BYTES);
        tma_load_plane(reinterpret_cast<float*>(smem + (q % NBUF) * T::PLANE_STRIDE), src_map, &bar[q % NBUF],
                       x0 - HX, y0 - 1, k0 - 1 + q);
    };
    auto wait = [&](int q) { return mbar_wait(&bar[q % NBUF], (uint32_t)((q / NBUF) & 1), err); };
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(&bar[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int issued = 0;                                     // meaningful in thread 0 only
    if (tid == 0)
        for (; issued < NBUF && issued < nplanes; ++issued) issue(issued);

    const int lane_x = tid % LX, row0 = tid / LX;
    const int32_t i0 = x0 + 4 * lane_x;
    const bool xin = i0 < nx;                           // nx % 4 == 0: all four or none
    const bool xlo = i0 == 0, xhi = i0 + 4 >= nx;
    const int sx = HX + 4 * lane_x;                     // shared column of the first voxel
    const int64_t plane = (int64_t)nx * ny;
    float4 below[RPT], cur[RPT];

    // Every wait is bounded and the go/stop decision after it is made
    // block-wide (__syncthreads_and), so a timeout can never leave part of the
    // block waiting at a barrier the rest has abandoned.
    int waited = 0;                                     // planes 0..waited-1 landed (all threads agree)
    bool ok = wait(0) & wait(1);
    ok = __syncthreads_and(ok);
    if (ok) {
        waited = 2;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            const int s = (row0 + r * T::ROWS + 1) * T::BXW + sx;
            cur[r] = *reinterpret_cast<const float4*>(buf(1) + s);
            below[r] = (k0 > 0) ? *reinterpret_cast<const float4*>(buf(0) + s) : ghost4(f, AGB_FACE_ZMIN, cur[r]);
        }
        ok = wait(2);                                   // nplanes >= 3
        fence_proxy_async_smem();                       // plane 0's slot is refilled next
        ok = __syncthreads_and(ok);                     // also: everyone is done with plane 0
        if (ok) {
            waited = 3;
            if (tid == 0 && issued < nplanes) issue(issued++);
        }
    }
    for (int32_t k = k0; k < k1 && ok; ++k) {
        const int q = k - k0 + 1;                       // plane of z = k; plane q + 1 has landed
        const float* pc = buf(q);
        const float* pa = buf(q + 1);
        const bool top = k == nz - 1;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            const int ty = row0 + r * T::ROWS;
            const int32_t j = y0 + ty;
            const int s = (ty + 1) * T::BXW + sx;
            const float4 c = cur[r];
            const float4 a = top ? ghost4(f, AGB_FACE_ZMAX, c) : *reinterpret_cast<const float4*>(pa + s);
            if (xin && j < ny) {
                const float4 d = (j > 0) ? *reinterpret_cast<const float4*>(pc + s - T::BXW)
                                         : ghost4(f, AGB_FACE_YMIN, c);
                const float4 u = (j < ny - 1) ? *reinterpret_cast<const float4*>(pc + s + T::BXW)
                                              : ghost4(f, AGB_FACE_YMAX, c);
                const float l = xlo ? ghost(f, AGB_FACE_XMIN, c.x) : pc[s - 1];
                const float rr = xhi ? ghost(f, AGB_FACE_XMAX, c.w) : pc[s + 4];
                const float4 b = below[r];
                float4 o;
                o.x = ftcs7(c.x, l, c.y, d.x, u.x, b.x, a.x, coeff);
                o.y = ftcs7(c.y, c.x, c.z, d.y, u.y, b.y, a.y, coeff);
                o.z = ftcs7(c.z, c.y, c.w, d.z, u.z, b.z, a.z, coeff);
                o.w = ftcs7(c.w, c.z, rr, d.w, u.w, b.w, a.w, coeff);
                *reinterpret_cast<float4*>(dst + (int64_t)k * plane + (int64_t)j * nx + i0) = o;
            }
            below[r] = c;
            cur[r] = a;
        }
        if (k + 1 < k1) {
            // Plane q + 2 is the next step's "above"; the barrier also marks
            // plane q as free, so its slot takes plane q + NBUF.
            ok = wait(q + 2);
            fence_proxy_async_smem();                   // plane q's slot is refilled next
            ok = __syncthreads_and(ok);
            if (ok) {
                waited = q + 3;
                if (tid == 0 && issued < nplanes) issue(issued++);
            }
        }
    }
    // A CTA that gave up waits (bounded) for its own copies still in flight
    // before leaving, so no transfer lands in shared memory after it exits.
    if (!ok && tid == 0)
        for (int q = waited; q < issued; ++q) (void)wait(q);
}

template <int LX, int RPT>
__global__ void __launch_bounds__(256) ftcs3d_tma_kernel(const __grid_constant__ CUtensorMap src_map,
                                                         float* __restrict__ dst, int32_t nx, int32_t ny,
                                                         int32_t nz, int32_t zc, float coeff, Faces f,
                                                         uint32_t* err, int32_t early_trigger) {
    pdl_wait();
    if (early_trigger) pdl_trigger();
    ftcs3d_tma_body<LX, RPT>(&src_map, dst, nx, ny, nz, zc, coeff, f, err, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Batched passes (agb_batch): chambers of equal grids and tiling, chamber
// blockIdx.z / zchunks. Each tensor map sits in a device table written before
// the launch; the issuing thread acquires it for the tensor-map proxy first.
template <int LX, int RPT>
__global__ void __launch_bounds__(256) ftcs3d_tma_batch(const FtcsChamber* __restrict__ tab, int32_t nx,
                                                        int32_t ny, int32_t nz, int32_t zc, int32_t zchunks) {
    pdl_wait();
    const int32_t ch = blockIdx.z / zchunks;
    const FtcsChamber& a = tab[ch];
    Faces f;
#pragma unroll
    for (int k = 0; k < 6; ++k) { f.bc[k] = a.bc[k]; f.val[k] = a.face[k]; }
    f.robin = a.robin;
    if (threadIdx.x == 0)
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&a.map) : "memory");
    ftcs3d_tma_body<LX, RPT>(&a.map, a.dst, nx, ny, nz, zc, a.coeff, f, a.err, blockIdx.x, blockIdx.y,
                             blockIdx.z - ch * zchunks);
}

// Sparse flush: every occupied cell exchanges its voxel's accumulator for zero;
// exactly one thread per voxel sees the nonzero sum and folds it in, so the
// result equals the reference's dense flush over all voxels (a voxel without a
// depositing cell holds zero). Optionally also zeroes a per-voxel demand
// accumulator of the same grid (the CO2 rationing buffer).
// The temperature flush (`gated`) is skipped while no cell has deposited heat
// since the last one (thermal_kernel_body raises S->t_deposited): with every
// deposit word zero the dense flush it replaces changes nothing either. All
// CTAs read the flag before any clears it: each counts itself done after its
// read, and the last one to finish clears the flag and the count.
// `vox`, when set, holds each cell's voxel in g (the thermal substeps' record).
__device__ __forceinline__ void flush_by_cells_kernel_body(DevState* S, const GridDev& g, unsigned long long* demand,
                                                           bool gated, const int32_t* vox, Blk blk) {
    if (gated && *(volatile const uint32_t*)&S->t_deposited == 0u) return;   // block-uniform
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS_B(i, blk, n) {
        if (!(v.flags[i] & AGB_FLAG_OCCUPIED)) continue;
        const int64_t idx = vox ? (int64_t)vox[i] : grid_nearest(g, (float)v.x[i], (float)v.y[i], (float)v.z[i]);
        const unsigned long long raw = atomicExch(&g.deposit[idx], 0ull);
        if (raw != 0ull)
            g.value[idx] = fa(g.value[idx], fixed_to_f((long long)raw, g.inv_scale_f, g.inv_scale_lo, g.scale));
        if (demand) demand[idx] = 0ull;
    }
    if (!gated) return;
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(&S->t_flush_fin, 1u) == (uint32_t)blk.n - 1u) {
        S->t_deposited = 0u;
        S->t_flush_fin = 0u;
    }
}

__global__ void flush_by_cells_kernel(DevState* S, GridDev g, unsigned long long* demand, int gated,
                                      const int32_t* vox) {
    pdl_wait();
    flush_by_cells_kernel_body(S, g, demand, gated != 0, vox, grid_blk());
}

AGB_BATCHED(flush_batch, 256, flush_by_cells_kernel_body(a.S, a.g, nullptr, true, a.c.t_vox, blk))

}  // namespace

bool launch_batched_grid(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, cudaStream_t s) {
    if (st != BStage::Flush) return false;
    launch_k(flush_batch, (unsigned)blocks, 256, 0, s, tab, map);
    return true;
}

void launch_fill(float* v, int64_t n, float value, cudaStream_t s) {
    const int64_t blocks = (n + 255) / 256;
    launch_k(fill_kernel, (unsigned)(blocks > 4096 ? 4096 : blocks), 256, 0, s, v, n, value);
}

void launch_brush(float* v, const GridDev& g, float cx, float cy, float radius, float amount,
                  int32_t x0, int32_t y0, int32_t bw, int32_t bh, cudaStream_t s) {
    const int64_t n = (int64_t)bw * bh * g.nz;
    if (n <= 0) return;
    const int64_t blocks = (n + 255) / 256;
    launch_k(brush_kernel, (unsigned)(blocks > 4096 ? 4096 : blocks), 256, 0, s, v, g, cx, cy, radius, amount,
             x0, y0, bw, bh);
}

namespace {

// Tilings of the TMA stencil: (lanes along x, rows per thread). Every tiling
// computes each voxel with the same operations, so the choice changes speed only.
template <int LX, int RPT>
struct TmaInstance {
    static void* fn() { return reinterpret_cast<void*>(&ftcs3d_tma_kernel<LX, RPT>); }
    static int slots_per_sm() {
        static int n = -1;
        if (n < 0) {
            cudaFuncSetAttribute(ftcs3d_tma_kernel<LX, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TmaTile<LX, RPT>::SMEM);
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ftcs3d_tma_kernel<LX, RPT>, 256,
                                                              TmaTile<LX, RPT>::SMEM) != cudaSuccess || b < 1)
                b = 1;
            n = b;
        }
        return n;
    }
    static void launch_batch(const FtcsChamber* tab, int32_t nch, int32_t nx, int32_t ny, int32_t nz, int32_t zc,
                             cudaStream_t s) {
        using T = TmaTile<LX, RPT>;
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(ftcs3d_tma_batch<LX, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM);
            attr = true;
        }
        const int32_t zchunks = (nz + zc - 1) / zc;
        const dim3 grid((nx + T::TXW - 1) / T::TXW, (ny + T::TYH - 1) / T::TYH, zchunks * nch);
        launch_k(ftcs3d_tma_batch<LX, RPT>, grid, 256, T::SMEM, s, tab, nx, ny, nz, zc, zchunks);
    }
    static cudaError_t launch(const GridDev& g, int zc, const CUtensorMap* map, float* dst, float coeff,
                              const Faces& f, uint32_t* err, cudaStream_t s) {
        using T = TmaTile<LX, RPT>;
        (void)slots_per_sm();                           // sets the shared-memory attribute once
        const dim3 grid((g.nx + T::TXW - 1) / T::TXW, (g.ny + T::TYH - 1) / T::TYH, (g.nz + zc - 1) / zc);
        // Letting the next pass's CTAs take free slots early paid on a 256^3
        // field (24.7 -> 21.5 us a pass) and cost on a 128^3 one (5.2 -> 5.7
        // us: its one short wave then lands unevenly over the SMs), so small
        // fields trigger at exit.
        const int32_t early = (int64_t)g.nx * g.ny * g.nz >= (int64_t)1 << 24;
        return launch_k(ftcs3d_tma_kernel<LX, RPT>, grid, 256, T::SMEM, s, *map, dst, g.nx, g.ny, g.nz, zc, coeff,
                        f, err, early);
    }
};

int sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

}  // namespace

// Tiling and z chunk of the TMA stencil for a grid. Rows 256 wide and wider
// use 32 lanes along x (a warp covers one 128-voxel row), narrower rows 16;
// grids under 8 M voxels take one row per thread (more CTAs), larger ones two.
// The z chunk is the smallest that fits the whole grid in one wave of resident
// CTAs (fewer planes per CTA re-read more halo planes), at least 2 planes.
// On a GB300 a pass on 256^3 takes 23.3 us inside a graph of passes (5.8 TB/s,
// 704 CTAs of 12 planes) and 8.2 us on 128^3, within 5 % of the best tiling
// of each. AGB_FTCS_TILE="lx,rpt,zc"
// overrides the choice (a tuning knob; results are the same for every tiling).
FtcsPlan ftcs_plan_with(int32_t nx, int32_t ny, int32_t nz, int32_t lx, int32_t rpt, int32_t zc_in) {
    return ftcs_plan_copies(nx, ny, nz, lx, rpt, zc_in, 1);
}

FtcsPlan ftcs_plan_copies(int32_t nx, int32_t ny, int32_t nz, int32_t lx, int32_t rpt, int32_t zc_in,
                          int32_t copies) {
    FtcsPlan p{lx, rpt, zc_in > 0 ? zc_in : 0};
    if (!(lx == 16 || lx == 32) || !(rpt == 1 || rpt == 2 || rpt == 4) || (lx == 16 && rpt == 4)) {
        p.lx = 16; p.rpt = 1;
    }
    if (copies < 1) copies = 1;
    if (p.zc == 0) {
        int per_sm = 1;
        if (p.lx == 32) per_sm = p.rpt == 1 ? TmaInstance<32, 1>::slots_per_sm()
                               : p.rpt == 2 ? TmaInstance<32, 2>::slots_per_sm() : TmaInstance<32, 4>::slots_per_sm();
        else per_sm = p.rpt == 1 ? TmaInstance<16, 1>::slots_per_sm() : TmaInstance<16, 2>::slots_per_sm();
        const int64_t tx = 4 * p.lx, ty = (256 / p.lx) * p.rpt;
        const int64_t tiles = ((nx + tx - 1) / tx) * ((ny + ty - 1) / ty);
        const int64_t slots = (int64_t)sm_count() * per_sm;
        // As many z chunks as one wave holds (rounding the chunk count up
        // instead would leave a few CTAs to run alone after the wave).
        const int64_t per_wave = slots / (tiles * copies);
        int64_t zc = per_wave >= 1 ? (nz + per_wave - 1) / per_wave : (tiles * nz * copies + slots - 1) / slots;
        zc = zc < 2 ? 2 : (zc > 32 ? 32 : zc);
        const int64_t chunks = (nz + zc - 1) / zc;
        p.zc = (int32_t)((nz + chunks - 1) / chunks);
    }
    return p;
}

FtcsPlan ftcs_plan(int32_t nx, int32_t ny, int32_t nz) {
    const int64_t voxels = (int64_t)nx * ny * nz;
    int32_t lx = nx >= 256 ? 32 : 16, rpt = voxels >= (8 << 20) ? 2 : 1, zc = 0;
    if (const char* e = std::getenv("AGB_FTCS_TILE")) {
        int a = 0, b = 0, c = 0;
        if (std::sscanf(e, "%d,%d,%d", &a, &b, &c) >= 2 && (a == 16 || a == 32) && (b == 1 || b == 2 || b == 4) &&
            !(a == 16 && b == 4)) {
            lx = a; rpt = b; zc = c > 0 ? c : 0;
        }
    }
    return ftcs_plan_with(nx, ny, nz, lx, rpt, zc);
}

cudaError_t launch_ftcs(const GridDev& g, const float* src, float* dst, float coeff, const int32_t* bc,
                        const float* face, float robin, const CUtensorMap* src_map, const FtcsPlan* plan,
                        uint32_t* err, cudaStream_t s) {
    Faces f;
    for (int k = 0; k < 6; ++k) { f.bc[k] = bc[k]; f.val[k] = face[k]; }
    f.robin = robin;
    if (g.nz > 1 && src_map != nullptr && plan != nullptr) {
        const FtcsPlan p = *plan;
        if (p.lx == 32) {
            if (p.rpt == 1) return TmaInstance<32, 1>::launch(g, p.zc, src_map, dst, coeff, f, err, s);
            if (p.rpt == 2) return TmaInstance<32, 2>::launch(g, p.zc, src_map, dst, coeff, f, err, s);
            return TmaInstance<32, 4>::launch(g, p.zc, src_map, dst, coeff, f, err, s);
        }
        if (p.rpt == 1) return TmaInstance<16, 1>::launch(g, p.zc, src_map, dst, coeff, f, err, s);
        return TmaInstance<16, 2>::launch(g, p.zc, src_map, dst, coeff, f, err, s);
    }
    const dim3 block(32, 8);
    if (g.nz == 1) {
        const dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8);
        return launch_k(ftcs2d_kernel, grid, block, 0, s, src, dst, g.nx, g.ny, coeff, f);
    }
    const dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + ZCHUNK - 1) / ZCHUNK);
    return launch_k(ftcs3d_kernel, grid, block, 0, s, src, dst, g.nx, g.ny, g.nz, coeff, f);
}

bool ftcs_plain_fits(int32_t nx, int32_t ny, int32_t nz) {
    if (nx < 1 || ny < 1 || nz < 1) return false;
    return (ny + 7) / 8 <= 65535 && (nz == 1 || (nz + ZCHUNK - 1) / ZCHUNK <= 65535);
}

void launch_ftcs_batch(const FtcsChamber* tab, int32_t nch, int32_t nx, int32_t ny, int32_t nz,
                       const FtcsPlan& p, cudaStream_t s) {
    if (nch <= 0) return;
    if (p.lx == 32) {
        if (p.rpt == 1) TmaInstance<32, 1>::launch_batch(tab, nch, nx, ny, nz, p.zc, s);
        else if (p.rpt == 2) TmaInstance<32, 2>::launch_batch(tab, nch, nx, ny, nz, p.zc, s);
        else TmaInstance<32, 4>::launch_batch(tab, nch, nx, ny, nz, p.zc, s);
    } else {
        if (p.rpt == 1) TmaInstance<16, 1>::launch_batch(tab, nch, nx, ny, nz, p.zc, s);
        else TmaInstance<16, 2>::launch_batch(tab, nch, nx, ny, nz, p.zc, s);
    }
}

void launch_flush_by_cells(DevState* S, GridDev g, unsigned long long* demand, int32_t grid_blocks,
                           cudaStream_t s, bool temperature, const int32_t* vox) {
    launch_k(flush_by_cells_kernel, grid_blocks, 256, 0, s, S, g, demand, temperature ? 1 : 0, vox);
}

}  // namespace agb

namespace agb {

// A 3-D tensor map over one field buffer for ftcs3d_tma_kernel, its box the
// tile (plus halo) of the grid's tiling: (4 lx + 8) x (256 / lx * rpt + 2) x 1
// floats. Returns false (plain kernel used instead) when the driver entry point
// is unavailable or the grid's row pitch is not a multiple of 16 bytes.
bool make_plane_map(CUtensorMap* map, float* base, int32_t nx, int32_t ny, int32_t nz, const FtcsPlan& p) {
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
    const cuuint32_t box[3] = {(cuuint32_t)(4 * p.lx + 2 * HX), (cuuint32_t)((256 / p.lx) * p.rpt + 2), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace agb
