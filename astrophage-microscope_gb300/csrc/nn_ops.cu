// nn_ops.cu -- the memory-bound layers of the field surrogate: layout
// transposes for the weight gradient, 2x average pooling and nearest
// upsampling with the skip connection (and their backward passes, which also
// apply the ReLU mask of the activation they feed), weight flips for the
// input gradient, and deterministic reductions. Arithmetic is FP32; tensors
// are BF16.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "nn.h"

namespace agb {
namespace nn {
namespace {

__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 tobf(float v) { return __float2bfloat16_rn(v); }

unsigned grid_for(int64_t n, int block = 256) {
    const int64_t b = (n + block - 1) / block;
    return (unsigned)(b < 65536 * 16 ? b : 65536 * 16);
}

// [m][c] -> [c][m] through a 32 x 33 shared tile.
__global__ void transpose_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ xt, int64_t m,
                                 int c) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int64_t mb = (int64_t)blockIdx.x * 32;
    const int cb = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t mm = mb + r;
        const int cc = cb + threadIdx.x;
        tile[r][threadIdx.x] = (mm < m && cc < c) ? x[mm * c + cc] : tobf(0.0f);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int cc = cb + r;
        const int64_t mm = mb + threadIdx.x;
        if (cc < c && mm < m) xt[(int64_t)cc * m + mm] = tile[threadIdx.x][r];
    }
}

// xt3[d][ch][z][y][x] = x[z][y][x + d - 1][ch] (zero outside the grid).
__global__ void shifted_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ xt3, int D, int H,
                               int W, int c) {
    const int64_t m = (int64_t)D * H * W;
    const int64_t total = 3 * (int64_t)c * m;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = i % m;
        const int64_t dc = i / m;
        const int ch = (int)(dc % c), d = (int)(dc / c);
        const int xx = (int)(v % W) + d - 1;
        xt3[i] = (xx >= 0 && xx < W) ? x[(v + d - 1) * c + ch] : tobf(0.0f);
    }
}

__global__ void reduce_kernel(const float* __restrict__ partial, float* __restrict__ dw, int splits, int64_t per_tap,
                              float scale, int accumulate) {
    const int64_t total = 27 * per_tap;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = i / per_tap, k = i % per_tap;
        const float* p = partial + t * splits * per_tap + k;
        float s = 0.0f;
        for (int j = 0; j < splits; ++j) s += p[(int64_t)j * per_tap];
        dw[i] = accumulate ? dw[i] + scale * s : scale * s;
    }
}

// Column sums of dy [m][c] in two fixed-order passes.
__global__ void colsum_partial_kernel(const __nv_bfloat16* __restrict__ dy, float* __restrict__ part, int64_t m,
                                      int c, int64_t rows_per) {
    const int col = threadIdx.x;
    if (col >= c) return;
    const int64_t r0 = blockIdx.x * rows_per;
    const int64_t r1 = r0 + rows_per < m ? r0 + rows_per : m;
    float s = 0.0f;
    for (int64_t r = r0; r < r1; ++r) s += bf(dy[r * c + col]);
    part[(int64_t)blockIdx.x * c + col] = s;
}
__global__ void colsum_final_kernel(const float* __restrict__ part, float* __restrict__ db, int blocks, int c) {
    const int col = threadIdx.x;
    if (col >= c) return;
    float s = 0.0f;
    for (int b = 0; b < blocks; ++b) s += part[(int64_t)b * c + col];
    db[col] = s;
}

// wf[26 - t][ci][co] = w[t][co][ci]
__global__ void flip_kernel(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wf, int cout, int cin) {
    const int64_t total = 27LL * cout * cin;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)(i / ((int64_t)cout * cin));
        const int r = (int)(i % ((int64_t)cout * cin));
        const int co = r / cin, ci = r % cin;
        wf[(int64_t)(26 - t) * cin * cout + (int64_t)ci * cout + co] = w[i];
    }
}

// Fine dims D, H, W (even); y is [D/2][H/2][W/2][c].
// Eight channels (16 bytes) per thread; per channel the same FP32 sum in the
// same order as one channel per thread would form it.
struct Bf8 {
    float v[8];
};
__device__ __forceinline__ Bf8 load8(const __nv_bfloat16* p) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
    Bf8 r;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]));
        r.v[2 * k] = f.x;
        r.v[2 * k + 1] = f.y;
    }
    return r;
}
__device__ __forceinline__ void store8(__nv_bfloat16* p, const Bf8& r) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(r.v[2 * k], r.v[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t*>(&h);
    }
    *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void avgpool_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int D, int H, int W,
                               int c) {
    const int d2 = D / 2, h2 = H / 2, w2 = W / 2, cq = c / 8;
    const int64_t total = (int64_t)d2 * h2 * w2 * cq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i % cq);
        const int v = (int)(i / cq);                 // coarse voxel (< 2^31)
        const int X = v % w2, Y = (v / w2) % h2, Z = v / (w2 * h2);
        Bf8 s;
#pragma unroll
        for (int j = 0; j < 8; ++j) s.v[j] = 0.0f;
        for (int k = 0; k < 8; ++k) {
            const int z = 2 * Z + (k >> 2), yy = 2 * Y + ((k >> 1) & 1), xx = 2 * X + (k & 1);
            const Bf8 a = load8(x + (((int64_t)z * H + yy) * W + xx) * c + q * 8);
#pragma unroll
            for (int j = 0; j < 8; ++j) s.v[j] += a.v[j];
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) s.v[j] = 0.125f * s.v[j];
        store8(y + (int64_t)v * c + q * 8, s);
    }
}

// dx (fine) = dskip + dy(parent) / 8, zeroed where act <= 0.
__global__ void avgpool_bwd_kernel(const __nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ dskip,
                                   const __nv_bfloat16* __restrict__ act, __nv_bfloat16* __restrict__ dx, int D, int H,
                                   int W, int c) {
    const int64_t total = (int64_t)D * H * W * c;
    const int h2 = H / 2, w2 = W / 2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        int64_t v = i / c;
        const int xx = (int)(v % W); v /= W;
        const int yy = (int)(v % H);
        const int z = (int)(v / H);
        float g = 0.125f * bf(dy[(((int64_t)(z / 2) * h2 + yy / 2) * w2 + xx / 2) * c + ch]);
        if (dskip) g += bf(dskip[i]);
        if (act && !(bf(act[i]) > 0.0f)) g = 0.0f;
        dx[i] = tobf(g);
    }
}

// y (fine) = coarse(parent) + skip.
__global__ void upsample_add_kernel(const __nv_bfloat16* __restrict__ coarse, const __nv_bfloat16* __restrict__ skip,
                                    __nv_bfloat16* __restrict__ y, int D, int H, int W, int c) {
    const int cq = c / 8, h2 = H / 2, w2 = W / 2;
    const int64_t total = (int64_t)D * H * W * cq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i % cq);
        const int v = (int)(i / cq);                 // fine voxel (< 2^31)
        const int xx = v % W, yy = (v / W) % H, z = v / (W * H);
        Bf8 s = load8(coarse + (((int64_t)(z / 2) * h2 + yy / 2) * w2 + xx / 2) * c + q * 8);
        if (skip) {
            const Bf8 k = load8(skip + (int64_t)v * c + q * 8);
#pragma unroll
            for (int j = 0; j < 8; ++j) s.v[j] += k.v[j];
        }
        store8(y + (int64_t)v * c + q * 8, s);
    }
}

// dcoarse = sum of the 8 children of dy, zeroed where act (coarse) <= 0.
// D, H, W are the coarse dims.
__global__ void upsample_bwd_kernel(const __nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ act,
                                    __nv_bfloat16* __restrict__ dc, int D, int H, int W, int c) {
    const int64_t total = (int64_t)D * H * W * c;
    const int H2 = 2 * H, W2 = 2 * W;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c);
        int64_t v = i / c;
        const int X = (int)(v % W); v /= W;
        const int Y = (int)(v % H);
        const int Z = (int)(v / H);
        float s = 0.0f;
        for (int k = 0; k < 8; ++k) {
            const int z = 2 * Z + (k >> 2), yy = 2 * Y + ((k >> 1) & 1), xx = 2 * X + (k & 1);
            s += bf(dy[(((int64_t)z * H2 + yy) * W2 + xx) * c + ch]);
        }
        if (act && !(bf(act[i]) > 0.0f)) s = 0.0f;
        dc[i] = tobf(s);
    }
}

}  // namespace

void to_channel_major(const __nv_bfloat16* x, __nv_bfloat16* xt, int64_t m, int c, cudaStream_t s) {
    const dim3 grid((unsigned)((m + 31) / 32), (unsigned)((c + 31) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(x, xt, m, c);
}
void to_channel_major_shifted(const __nv_bfloat16* x, __nv_bfloat16* xt3, int D, int H, int W, int c,
                              cudaStream_t s) {
    shifted_kernel<<<grid_for(3LL * c * D * H * W), 256, 0, s>>>(x, xt3, D, H, W, c);
}
void reduce_partials(const float* partial, float* dw, int splits, int64_t per_tap, float scale, int accumulate,
                     cudaStream_t s) {
    reduce_kernel<<<grid_for(27 * per_tap), 256, 0, s>>>(partial, dw, splits, per_tap, scale, accumulate);
}
void bias_grad(const __nv_bfloat16* dy, float* db, int64_t m, int c, float* scratch, cudaStream_t s) {
    const int blocks = 1024;
    const int64_t rows_per = (m + blocks - 1) / blocks;
    colsum_partial_kernel<<<blocks, 128, 0, s>>>(dy, scratch, m, c, rows_per);
    colsum_final_kernel<<<1, 128, 0, s>>>(scratch, db, blocks, c);
}
void flip_weights(const __nv_bfloat16* w, __nv_bfloat16* wf, int cout, int cin, cudaStream_t s) {
    flip_kernel<<<grid_for(27LL * cout * cin), 256, 0, s>>>(w, wf, cout, cin);
}
void avgpool2(const __nv_bfloat16* x, __nv_bfloat16* y, int D, int H, int W, int c, cudaStream_t s) {
    avgpool_kernel<<<grid_for((int64_t)D * H * W * c / 64), 256, 0, s>>>(x, y, D, H, W, c);
}
void avgpool2_backward_add(const __nv_bfloat16* dy, const __nv_bfloat16* dskip, const __nv_bfloat16* act,
                           __nv_bfloat16* dx, int D, int H, int W, int c, cudaStream_t s) {
    avgpool_bwd_kernel<<<grid_for((int64_t)D * H * W * c), 256, 0, s>>>(dy, dskip, act, dx, D, H, W, c);
}
void upsample2_add(const __nv_bfloat16* coarse, const __nv_bfloat16* skip, __nv_bfloat16* y, int D, int H, int W,
                   int c, cudaStream_t s) {
    upsample_add_kernel<<<grid_for((int64_t)D * H * W * c / 8), 256, 0, s>>>(coarse, skip, y, D, H, W, c);
}
void upsample2_backward(const __nv_bfloat16* dy, const __nv_bfloat16* act, __nv_bfloat16* dcoarse, int D, int H,
                        int W, int c, cudaStream_t s) {
    upsample_bwd_kernel<<<grid_for((int64_t)D * H * W * c), 256, 0, s>>>(dy, act, dcoarse, D, H, W, c);
}

}  // namespace nn
}  // namespace agb
