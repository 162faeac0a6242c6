// k_grid.cu -- FTCS conduction/diffusion and the fixed-point flush.
//
// HBM-bound: a pass reads each voxel once and writes it once (8 B per
// voxel-step). The 3-D kernel marches each thread up a z column keeping the
// below/centre/above values in registers, so every plane is fetched once from
// DRAM; in-plane neighbours come from L1. Arithmetic follows
// src/fields/diffuse.cu:19-44 operation for operation (explicitly rounded, no
// contraction), so nz == 1 reproduces the reference bit for bit.
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
                 const float* face, float robin, cudaStream_t s) {
    Faces f;
    for (int k = 0; k < 6; ++k) { f.bc[k] = bc[k]; f.val[k] = face[k]; }
    f.robin = robin;
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
