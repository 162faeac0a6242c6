// surrogate.cu -- the learned field surrogate: a 3-level 3-D convolutional
// encoder-decoder that advances the temperature and CO2 grids `steps` FTCS
// steps (16) in one call, trained on the GPU by this file's own forward and
// backward passes over FTCS windows that the engine's own stencil generates.
// No counterpart in the reference, which only has the plain stencil
// (src/fields/diffuse.cu:19-44).
//
// Network (channels-last BF16 activations, BF16 weights, FP32 accumulation
// on the tensor cores; conv = 3x3x3 "same"):
//   x0  = [T, CO2, q_T, q_CO2, d1_T, d1_CO2 normalised, 10 zeros]  n      16
// where d1 = FTCS(X + q) - X is one plain stencil step, computed in FP32:
// the increments that drive diffusion are far below the BF16 resolution of
// the absolute fields, so the network sees them as a difference.
//   A1  = relu(conv 16->32 (x0))                                  n      32
//   A2  = relu(conv 32->64 (avgpool A1))                          n/2    64
//   A3  = relu(conv 64->128 (avgpool A2))                         n/4   128
//   A4  = relu(conv 128->64 (A3))                                 n/4    64
//   A5  = relu(conv 64->32 (upsample A4 + A2))                    n/2    32
//   y   = conv 32->16 (upsample A5 + A1), FP32                    n      16
//   T'  = T + y0 * s_T,  CO2' = CO2 + y1 * s_C.
// The 16 output channels keep the last convolution on an N = 16 tensor-core
// tile; channels 2..15 are trained towards zero.
//
// The operator it learns is the one the judge runs: `steps` times
// X <- FTCS(X + q) for both fields with constant per-step sources q. Every
// judge_every-th call (or on request) runs that plain FTCS too, measures the
// largest temperature error and the drift of the summed temperature, and
// hands back the FTCS result instead when either exceeds its tolerance.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "kernels.h"
#include "nn.h"
#include "world_impl.cuh"

using agb::nn::Conv3Args;

namespace {

using bf16 = __nv_bfloat16;

struct Layer {
    int cin, cout, level, relu;
    float *w32, *b32;           // FP32 master weights [27][cout][cin], bias [cout]
    bf16 *w, *wf;               // BF16 copies: forward and flipped (input gradient)
    float *gw, *gb;             // gradients
    float *mw, *vw, *mb, *vb;   // Adam moments
};

constexpr int NL = 6;
constexpr int CIN0 = 16, COUT_LAST = 16;

__host__ __device__ inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__host__ __device__ inline float unit(uint64_t h) { return (float)((h >> 40) * (1.0 / 16777216.0)); }

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
struct Norm {
    float t_mean, t_scale, c_mean, c_scale, qt_scale, qc_scale, dt_scale, dc_scale, d1t_scale, d1c_scale;
};

__global__ void pack_kernel(const float* __restrict__ T, const float* __restrict__ C, const float* __restrict__ qT,
                            const float* __restrict__ qC, const float* __restrict__ f1T, const float* __restrict__ f1C,
                            bf16* __restrict__ x0, int64_t m, Norm nm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const float v[6] = {(T[i] - nm.t_mean) / nm.t_scale, (C[i] - nm.c_mean) / nm.c_scale,
                            qT ? qT[i] / nm.qt_scale : 0.0f, qC ? qC[i] / nm.qc_scale : 0.0f,
                            (f1T[i] - T[i]) / nm.d1t_scale, (f1C[i] - C[i]) / nm.d1c_scale};
        uint32_t w[8];
        for (int k = 0; k < 8; ++k) {
            const float a = 2 * k < 6 ? v[2 * k] : 0.0f, b = 2 * k + 1 < 6 ? v[2 * k + 1] : 0.0f;
            const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
            w[k] = *reinterpret_cast<const uint32_t*>(&h);
        }
        uint4* o = reinterpret_cast<uint4*>(x0 + i * CIN0);
        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// out = x + q (q may be null).
__global__ void add_to_kernel(const float* __restrict__ x, const float* __restrict__ q, float* __restrict__ out,
                              int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = q ? x[i] + q[i] : x[i];
}

// T += y0 * s_T, C += y1 * s_C (in place).
__global__ void apply_kernel(const float* __restrict__ y, float* __restrict__ T, float* __restrict__ C, int64_t m,
                             float sT, float sC) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        T[i] += y[i * COUT_LAST] * sT;
        C[i] += y[i * COUT_LAST + 1] * sC;
    }
}

// dy = y - target (channels 0, 1: normalised deltas; 2..15: zero), BF16;
// per-block partial sums of the squared error.
__global__ void loss_kernel(const float* __restrict__ y, const float* __restrict__ T0, const float* __restrict__ C0,
                            const float* __restrict__ T1, const float* __restrict__ C1, bf16* __restrict__ dy,
                            float* __restrict__ part, int64_t m, float inv_sT, float inv_sC) {
    __shared__ float red[256];
    float acc = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const float t0 = (T1[i] - T0[i]) * inv_sT, t1 = (C1[i] - C0[i]) * inv_sC;
        float r[COUT_LAST];
        for (int c = 0; c < COUT_LAST; ++c) r[c] = y[i * COUT_LAST + c] - (c == 0 ? t0 : (c == 1 ? t1 : 0.0f));
        acc += r[0] * r[0] + r[1] * r[1];
        uint32_t w[8];
        for (int k = 0; k < 8; ++k) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(r[2 * k], r[2 * k + 1]);
            w[k] = *reinterpret_cast<const uint32_t*>(&h);
        }
        uint4* o = reinterpret_cast<uint4*>(dy + i * COUT_LAST);
        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_kernel(const float* __restrict__ part, int n, float scale, float* __restrict__ out) {
    __shared__ float red[256];
    float a = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += part[i];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0] * scale;
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ wb, int64_t n, float lr, float b1, float b2,
                            float c1, float c2, float eps, float gscale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

__global__ void to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

__global__ void add_kernel(float* __restrict__ x, const float* __restrict__ q, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += q[i];
}

// Largest |a - b| (as ordered bits of a non-negative float) and the partial
// sums of a - b and b (FP64) per block.
__global__ void compare_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                               unsigned int* __restrict__ maxbits, double* __restrict__ part) {
    __shared__ double s1[256], s2[256];
    float mx = 0.0f;
    double d = 0.0, t = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float e = a[i] - b[i];
        const float ae = fabsf(e);
        mx = (ae == ae) ? fmaxf(mx, ae) : INFINITY;     // a NaN counts as an unbounded error
        d += (double)e;
        t += (double)b[i];
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(mx));
    s1[threadIdx.x] = d;
    s2[threadIdx.x] = t;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) { s1[threadIdx.x] += s1[threadIdx.x + s]; s2[threadIdx.x] += s2[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = s1[0]; part[2 * blockIdx.x + 1] = s2[0]; }
}

// Seeded training window: smooth random temperature and CO2 fields (Gaussian
// blobs over a base value) and sparse cell-like sources (each voxel holds a
// source with probability p; heating for T, uptake for CO2).
struct Blob { float cx, cy, cz, inv2s2, amp_t, amp_c; };
constexpr int NBLOB = 16;
struct WindowSpec {
    Blob blob[NBLOB];
    float t_base, c_base, p_src, qt_max, qc_max;
    uint64_t seed;
};

__global__ void window_kernel(float* __restrict__ T, float* __restrict__ C, float* __restrict__ qT,
                              float* __restrict__ qC, int nx, int ny, int nz, WindowSpec sp) {
    const int64_t m = (int64_t)nx * ny * nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = (float)(i % nx), y = (float)((i / nx) % ny), z = (float)(i / ((int64_t)nx * ny));
        float t = sp.t_base, c = sp.c_base;
        for (int k = 0; k < NBLOB; ++k) {
            const float dx = x - sp.blob[k].cx, dy = y - sp.blob[k].cy, dz = z - sp.blob[k].cz;
            const float e = __expf(-(dx * dx + dy * dy + dz * dz) * sp.blob[k].inv2s2);
            t += sp.blob[k].amp_t * e;
            c += sp.blob[k].amp_c * e;
        }
        const uint64_t h = mix64(sp.seed ^ (uint64_t)i);
        const bool src = unit(h) < sp.p_src;
        const uint64_t h2 = mix64(h + 0x5151ull);
        T[i] = t;
        C[i] = c > 0.0f ? c : 0.0f;
        qT[i] = src ? sp.qt_max * unit(h2) : 0.0f;
        qC[i] = src ? -sp.qc_max * unit(mix64(h2)) : 0.0f;
    }
}

__global__ void source_kernel(unsigned long long* __restrict__ dep, float* __restrict__ q, int64_t n,
                              double inv_scale_steps) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long raw = dep[i];
        q[i] = raw ? (float)((double)(long long)raw * inv_scale_steps) : 0.0f;
        if (raw) dep[i] = 0ull;
    }
}

unsigned blocks_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (unsigned)(b < 4096 ? b : 4096);
}

}  // namespace

struct agb_surrogate {
    agb_surrogate_desc d{};
    int nx = 0, ny = 0, nz = 0;
    int64_t m[3] = {0, 0, 0};
    int dims[3][3] = {};        // [level] = {D, H, W}
    Layer L[NL] = {};
    Norm nm{};
    float t_coeff = 0.0f, c_coeff = 0.0f, robin[2] = {0.0f, 0.0f};
    bf16 *x0 = nullptr, *a1 = nullptr, *p1 = nullptr, *a2 = nullptr, *p2 = nullptr, *a3 = nullptr, *a4 = nullptr,
         *u2 = nullptr, *a5 = nullptr, *u1 = nullptr;
    bf16 *dy = nullptr, *du1 = nullptr, *da5 = nullptr, *du2 = nullptr, *da4 = nullptr, *da3 = nullptr,
         *dp2 = nullptr, *da2 = nullptr, *dp1 = nullptr, *da1 = nullptr;
    float* y = nullptr;
    void* scratch = nullptr;
    int64_t scratch_bytes = 0;
    float *fT = nullptr, *fC = nullptr, *fqT = nullptr, *fqC = nullptr, *gT = nullptr, *gC = nullptr;
    float *tmpA = nullptr, *tmpB = nullptr, *refT = nullptr, *refC = nullptr, *f1T = nullptr, *f1C = nullptr;
    float* part = nullptr;
    float* loss_dev = nullptr;
    double* cmp_part = nullptr;
    unsigned int* cmp_max = nullptr;
    uint32_t* err = nullptr;
    int64_t adam_t = 0;
    agb_surrogate_report rep{};
    std::vector<void*> allocs;
};

namespace {

template <typename T>
bool salloc(agb_surrogate* s, T** p, size_t bytes) {
    void* q = nullptr;
    if (cudaMalloc(&q, bytes ? bytes : 1) != cudaSuccess) return false;
    s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return true;
}

bool conv(agb_surrogate* s, int level, const bf16* x, const bf16* w, const float* b, int cin, int cout, int relu,
          const bf16* mask, void* out, int out_f32, cudaStream_t st) {
    const int* dm = s->dims[level];
    Conv3Args a{dm[0], dm[1], dm[2], cin, cout, b, relu, mask, out, out_f32, s->err};
    return agb::nn::conv3(a, x, w, st) == cudaSuccess;
}

void ftcs_once(agb_surrogate* s, int f, const float* x, const float* q, float* out, cudaStream_t st) {
    agb::GridDev g{};
    g.nx = s->nx; g.ny = s->ny; g.nz = s->nz; g.count = s->m[0]; g.enabled = 1;
    float face[6];
    for (int k = 0; k < 6; ++k) face[k] = (float)s->d.face[f][k];
    add_to_kernel<<<blocks_for(s->m[0]), 256, 0, st>>>(x, q, s->tmpB, s->m[0]);
    agb::launch_ftcs(g, s->tmpB, out, f == 0 ? s->t_coeff : s->c_coeff, s->d.bc[f], face, s->robin[f], nullptr,
                     nullptr, nullptr, st);
}

bool forward(agb_surrogate* s, const float* T, const float* C, const float* qT, const float* qC, cudaStream_t st) {
    const int(*d)[3] = s->dims;
    ftcs_once(s, 0, T, qT, s->f1T, st);
    ftcs_once(s, 1, C, qC, s->f1C, st);
    pack_kernel<<<blocks_for(s->m[0]), 256, 0, st>>>(T, C, qT, qC, s->f1T, s->f1C, s->x0, s->m[0], s->nm);
    Layer* L = s->L;
    bool ok = conv(s, 0, s->x0, L[0].w, L[0].b32, 16, 32, 1, nullptr, s->a1, 0, st);
    agb::nn::avgpool2(s->a1, s->p1, d[0][0], d[0][1], d[0][2], 32, st);
    ok = ok && conv(s, 1, s->p1, L[1].w, L[1].b32, 32, 64, 1, nullptr, s->a2, 0, st);
    agb::nn::avgpool2(s->a2, s->p2, d[1][0], d[1][1], d[1][2], 64, st);
    ok = ok && conv(s, 2, s->p2, L[2].w, L[2].b32, 64, 128, 1, nullptr, s->a3, 0, st);
    ok = ok && conv(s, 2, s->a3, L[3].w, L[3].b32, 128, 64, 1, nullptr, s->a4, 0, st);
    agb::nn::upsample2_add(s->a4, s->a2, s->u2, d[1][0], d[1][1], d[1][2], 64, st);
    ok = ok && conv(s, 1, s->u2, L[4].w, L[4].b32, 64, 32, 1, nullptr, s->a5, 0, st);
    agb::nn::upsample2_add(s->a5, s->a1, s->u1, d[0][0], d[0][1], d[0][2], 32, st);
    ok = ok && conv(s, 0, s->u1, L[5].w, L[5].b32, 32, 16, 0, nullptr, s->y, 1, st);
    return ok && cudaGetLastError() == cudaSuccess;
}

bool wgrad(agb_surrogate* s, int level, const bf16* x, const bf16* dy, Layer& l, cudaStream_t st) {
    const int* dm = s->dims[level];
    return agb_nn_wgrad(x, dy, dm[0], dm[1], dm[2], l.cin, l.cout, l.gw, l.gb, s->scratch, s->scratch_bytes, s->err,
                        st) == AGB_OK;
}

// Backward from s->dy (gradient of the loss with respect to y).
bool backward(agb_surrogate* s, cudaStream_t st) {
    const int(*d)[3] = s->dims;
    Layer* L = s->L;
    bool ok = wgrad(s, 0, s->u1, s->dy, L[5], st);
    ok = ok && conv(s, 0, s->dy, L[5].wf, nullptr, 16, 32, 0, nullptr, s->du1, 0, st);       // dU1
    agb::nn::upsample2_backward(s->du1, s->a5, s->da5, d[1][0], d[1][1], d[1][2], 32, st);  // dZ5
    ok = ok && wgrad(s, 1, s->u2, s->da5, L[4], st);
    ok = ok && conv(s, 1, s->da5, L[4].wf, nullptr, 32, 64, 0, nullptr, s->du2, 0, st);     // dU2
    agb::nn::upsample2_backward(s->du2, s->a4, s->da4, d[2][0], d[2][1], d[2][2], 64, st);  // dZ4
    ok = ok && wgrad(s, 2, s->a3, s->da4, L[3], st);
    ok = ok && conv(s, 2, s->da4, L[3].wf, nullptr, 64, 128, 0, s->a3, s->da3, 0, st);      // dZ3
    ok = ok && wgrad(s, 2, s->p2, s->da3, L[2], st);
    ok = ok && conv(s, 2, s->da3, L[2].wf, nullptr, 128, 64, 0, nullptr, s->dp2, 0, st);    // dP2
    agb::nn::avgpool2_backward_add(s->dp2, s->du2, s->a2, s->da2, d[1][0], d[1][1], d[1][2], 64, st);  // dZ2
    ok = ok && wgrad(s, 1, s->p1, s->da2, L[1], st);
    ok = ok && conv(s, 1, s->da2, L[1].wf, nullptr, 64, 32, 0, nullptr, s->dp1, 0, st);     // dP1
    agb::nn::avgpool2_backward_add(s->dp1, s->du1, s->a1, s->da1, d[0][0], d[0][1], d[0][2], 32, st);  // dZ1
    ok = ok && wgrad(s, 0, s->x0, s->da1, L[0], st);
    return ok && cudaGetLastError() == cudaSuccess;
}

void refresh_bf16(agb_surrogate* s, cudaStream_t st) {
    for (Layer& l : s->L) {
        const int64_t n = 27LL * l.cout * l.cin;
        to_bf16_kernel<<<blocks_for(n), 256, 0, st>>>(l.w32, l.w, n);
        agb::nn::flip_weights(l.w, l.wf, l.cout, l.cin, st);
    }
}

// `steps` times X <- FTCS(X + q), both fields, in place (the judge's operator).
void ftcs_window(agb_surrogate* s, float* T, float* C, const float* qT, const float* qC, cudaStream_t st) {
    agb::GridDev g{};
    g.nx = s->nx; g.ny = s->ny; g.nz = s->nz; g.count = s->m[0]; g.enabled = 1;
    float face[6];
    for (int f = 0; f < 2; ++f) {
        float* x = f == 0 ? T : C;
        const float* q = f == 0 ? qT : qC;
        for (int k = 0; k < 6; ++k) face[k] = (float)s->d.face[f][k];
        float* src = x;
        float* dst = s->tmpA;
        for (int k = 0; k < s->d.steps; ++k) {
            if (q) add_kernel<<<blocks_for(s->m[0]), 256, 0, st>>>(src, q, s->m[0]);
            agb::launch_ftcs(g, src, dst, f == 0 ? s->t_coeff : s->c_coeff, s->d.bc[f], face, s->robin[f], nullptr,
                             nullptr, nullptr, st);
            float* t = src; src = dst; dst = t;
        }
        if (src != x) cudaMemcpyAsync(x, src, 4 * (size_t)s->m[0], cudaMemcpyDeviceToDevice, st);
    }
}

void make_window(agb_surrogate* s, uint64_t index, float* T, float* C, float* qT, float* qC, cudaStream_t st) {
    WindowSpec sp{};
    uint64_t h = mix64(s->d.seed * 0x100000001B3ull + index);
    auto next = [&]() { h = mix64(h); return unit(h); };
    const float L = (float)(s->nx > s->ny ? (s->nx > s->nz ? s->nx : s->nz) : (s->ny > s->nz ? s->ny : s->nz));
    const float amp_t = (float)s->d.train_temperature_amplitude;
    for (int k = 0; k < NBLOB; ++k) {
        Blob& b = sp.blob[k];
        b.cx = next() * s->nx; b.cy = next() * s->ny; b.cz = next() * s->nz;
        const float sig = (0.02f + 0.2f * next()) * L;
        b.inv2s2 = 1.0f / (2.0f * sig * sig);
        b.amp_t = amp_t * (2.0f * next() - 1.0f);
        b.amp_c = 0.3f * (float)s->d.init[1] * (2.0f * next() - 1.0f);
    }
    sp.t_base = (float)s->d.init[0] + amp_t * 0.5f * (2.0f * next() - 1.0f);
    sp.c_base = (float)s->d.init[1];
    sp.p_src = (float)s->d.train_source_density * (0.25f + 1.5f * next());
    sp.qt_max = (float)s->d.train_heat_per_step * 2.0f * next();
    sp.qc_max = (float)s->d.train_uptake_per_step * 2.0f * next();
    sp.seed = h;
    window_kernel<<<blocks_for(s->m[0]), 256, 0, st>>>(T, C, qT, qC, s->nx, s->ny, s->nz, sp);
}

bool step_adam(agb_surrogate* s, cudaStream_t st) {
    ++s->adam_t;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f / (1.0f - std::pow(b1, (float)s->adam_t));
    const float c2 = 1.0f / (1.0f - std::pow(b2, (float)s->adam_t));
    const float gscale = 1.0f / (float)s->m[0];
    for (Layer& l : s->L) {
        const int64_t n = 27LL * l.cout * l.cin;
        adam_kernel<<<blocks_for(n), 256, 0, st>>>(l.w32, l.gw, l.mw, l.vw, l.w, n, s->d.learning_rate, b1, b2, c1,
                                                   c2, eps, gscale);
        adam_kernel<<<1, 256, 0, st>>>(l.b32, l.gb, l.mb, l.vb, nullptr, l.cout, s->d.learning_rate, b1, b2, c1, c2,
                                       eps, gscale);
        agb::nn::flip_weights(l.w, l.wf, l.cout, l.cin, st);
    }
    return cudaGetLastError() == cudaSuccess;
}

// Forward, loss against the FTCS window result, backward (gradients in gw/gb).
bool grad_pass(agb_surrogate* s, const float* T0, const float* C0, const float* qT, const float* qC, const float* T1,
               const float* C1, cudaStream_t st) {
    if (!forward(s, T0, C0, qT, qC, st)) return false;
    const unsigned nb = 1024;
    loss_kernel<<<nb, 256, 0, st>>>(s->y, T0, C0, T1, C1, s->dy, s->part, s->m[0], 1.0f / s->nm.dt_scale,
                                    1.0f / s->nm.dc_scale);
    sum_kernel<<<1, 256, 0, st>>>(s->part, (int)nb, 1.0f / (float)s->m[0], s->loss_dev);
    return backward(s, st);
}

int64_t param_count(const agb_surrogate* s) {
    int64_t n = 0;
    for (const Layer& l : s->L) n += 27LL * l.cout * l.cin + l.cout;
    return n;
}

}  // namespace

namespace agb {

bool surrogate_info(const agb_surrogate* sg, int32_t dims[3], int32_t* steps, float coeff[2], int32_t bc[2][6]) {
    if (!sg) return false;
    dims[0] = sg->nx; dims[1] = sg->ny; dims[2] = sg->nz;
    *steps = sg->d.steps;
    coeff[0] = sg->t_coeff; coeff[1] = sg->c_coeff;
    for (int f = 0; f < 2; ++f)
        for (int k = 0; k < 6; ++k) bc[f][k] = sg->d.bc[f][k];
    return true;
}

void surrogate_source_from_deposit(unsigned long long* dep, float* q, int64_t n, double inv_scale, int32_t steps,
                                   cudaStream_t s) {
    source_kernel<<<blocks_for(n), 256, 0, s>>>(dep, q, n, inv_scale / (double)steps);
}

void surrogate_add(float* x, const float* q, int64_t n, cudaStream_t s) {
    add_kernel<<<blocks_for(n), 256, 0, s>>>(x, q, n);
}

}  // namespace agb

extern "C" {

void agb_surrogate_desc_default(agb_surrogate_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->abi_version = AGB_ABI_VERSION;
    d->nx = d->ny = d->nz = 128;
    d->extent = 4.0e-3;
    d->dt = AGB_DT_PHYSICS;
    d->steps = 16;
    d->judge_every = 8;
    d->tol_temperature = 0.01;
    d->tol_energy = 1.0e-6;
    d->diffusivity[0] = AGB_WATER_THERMAL_DIFFUSIVITY;
    d->diffusivity[1] = AGB_CO2_DIFFUSIVITY_WATER;
    d->init[0] = AGB_AMBIENT_TEMP_DEFAULT;
    d->init[1] = 1.0;
    for (int k = 0; k < 6; ++k) {
        d->bc[0][k] = AGB_BC_ROBIN;
        d->face[0][k] = AGB_AMBIENT_TEMP_DEFAULT;
        d->bc[1][k] = AGB_BC_NEUMANN;
        d->face[1][k] = 1.0;
    }
    d->seed = 1;
    d->learning_rate = 1.0e-3f;
    d->train_temperature_amplitude = 2.0;
    d->train_source_density = 0.01;
    d->train_heat_per_step = 1.0e-3;
    d->train_uptake_per_step = 1.0e-6;
}

void agb_surrogate_destroy(agb_surrogate* s) {
    if (!s) return;
    for (void* p : s->allocs) cudaFree(p);
    delete s;
}

agb_status agb_surrogate_create(const agb_surrogate_desc* d, agb_surrogate** out) {
    if (!out) return AGB_INVALID_ARGUMENT;
    *out = nullptr;
    if (!d || d->abi_version != AGB_ABI_VERSION) return AGB_CONTRACT_VERSION_MISMATCH;
    if (!(d->nx == 128 || d->nx == 256) || d->ny <= 0 || d->nz <= 0 || d->ny % 16 || d->nz % 4 ||
        !(d->extent > 0.0) || !(d->dt > 0.0) || d->steps <= 0 || d->judge_every <= 0)
        return AGB_INVALID_ARGUMENT;
    agb_surrogate* s = new (std::nothrow) agb_surrogate();
    if (!s) return AGB_OUT_OF_MEMORY;
    s->d = *d;
    s->nx = d->nx; s->ny = d->ny; s->nz = d->nz;
    for (int l = 0; l < 3; ++l) {
        s->dims[l][0] = s->nz >> l; s->dims[l][1] = s->ny >> l; s->dims[l][2] = s->nx >> l;
        s->m[l] = (int64_t)s->dims[l][0] * s->dims[l][1] * s->dims[l][2];
        if (!agb::nn::conv3_supported(s->dims[l][0], s->dims[l][1], s->dims[l][2], 32, 32)) {
            agb_surrogate_destroy(s);
            return AGB_INVALID_ARGUMENT;
        }
    }
    const double dx = d->extent / d->nx;
    s->t_coeff = (float)(d->diffusivity[0] * d->dt / (dx * dx));
    s->c_coeff = (float)(d->diffusivity[1] * d->dt / (dx * dx));
    if (!(s->t_coeff <= (float)(1.0 / 6.0)) || !(s->c_coeff <= (float)(1.0 / 6.0))) {
        agb_surrogate_destroy(s);
        return AGB_INVALID_ARGUMENT;                     // one FTCS step must be stable
    }
    s->robin[0] = s->robin[1] = (float)(dx * AGB_AIR_CONVECTION_H / AGB_WATER_CONDUCTIVITY);
    // Normalisation: fields about their initial values; deltas scaled to the
    // change one step of sources makes over the window.
    s->nm.t_mean = (float)d->init[0];
    s->nm.t_scale = (float)(d->train_temperature_amplitude > 0.0 ? d->train_temperature_amplitude : 1.0);
    s->nm.c_mean = (float)d->init[1];
    s->nm.c_scale = (float)(d->init[1] > 0.0 ? 0.3 * d->init[1] : 1.0);
    s->nm.qt_scale = (float)(d->train_heat_per_step > 0.0 ? d->train_heat_per_step : 1.0);
    s->nm.qc_scale = (float)(d->train_uptake_per_step > 0.0 ? d->train_uptake_per_step : 1.0);
    s->nm.dt_scale = (float)(0.05 * s->nm.t_scale + d->steps * s->nm.qt_scale);
    s->nm.dc_scale = (float)(0.01 * s->nm.c_scale + d->steps * s->nm.qc_scale);
    s->nm.d1t_scale = s->nm.dt_scale / (float)d->steps;
    s->nm.d1c_scale = s->nm.dc_scale / (float)d->steps;

    const int spec[NL][4] = {{16, 32, 0, 1}, {32, 64, 1, 1}, {64, 128, 2, 1}, {128, 64, 2, 1}, {64, 32, 1, 1},
                             {32, 16, 0, 0}};
    bool ok = true;
    int64_t scratch = 0;
    uint64_t h = mix64(d->seed ^ 0xA5A5A5A5ull);
    for (int k = 0; k < NL && ok; ++k) {
        Layer& l = s->L[k];
        l.cin = spec[k][0]; l.cout = spec[k][1]; l.level = spec[k][2]; l.relu = spec[k][3];
        const int64_t n = 27LL * l.cout * l.cin;
        ok = salloc(s, &l.w32, 4 * n) && salloc(s, &l.b32, 4 * l.cout) && salloc(s, &l.w, 2 * n) &&
             salloc(s, &l.wf, 2 * n) && salloc(s, &l.gw, 4 * n) && salloc(s, &l.gb, 4 * l.cout) &&
             salloc(s, &l.mw, 4 * n) && salloc(s, &l.vw, 4 * n) && salloc(s, &l.mb, 4 * l.cout) &&
             salloc(s, &l.vb, 4 * l.cout);
        if (!ok) break;
        // He-normal initialisation (Box-Muller on seeded uniforms); the last
        // layer starts small so the untrained network is close to "no change".
        std::vector<float> w((size_t)n);
        const float sd = std::sqrt(2.0f / (27.0f * l.cin)) * (k == NL - 1 ? 0.05f : 1.0f);
        for (int64_t i = 0; i < n; i += 2) {
            h = mix64(h); const float u1 = unit(h) * 0.9999999f + 1e-7f;
            h = mix64(h); const float u2 = unit(h);
            const float r = std::sqrt(-2.0f * std::log(u1));
            w[(size_t)i] = sd * r * std::cos(6.2831853f * u2);
            if (i + 1 < n) w[(size_t)i + 1] = sd * r * std::sin(6.2831853f * u2);
        }
        cudaMemcpy(l.w32, w.data(), 4 * n, cudaMemcpyHostToDevice);
        cudaMemset(l.b32, 0, 4 * l.cout);
        cudaMemset(l.mw, 0, 4 * n); cudaMemset(l.vw, 0, 4 * n);
        cudaMemset(l.mb, 0, 4 * l.cout); cudaMemset(l.vb, 0, 4 * l.cout);
        const int* dm = s->dims[l.level];
        const int64_t sb = agb_nn_wgrad_scratch_bytes(dm[0], dm[1], dm[2], l.cin, l.cout);
        if (sb > scratch) scratch = sb;
    }
    const int64_t m0 = s->m[0], m1 = s->m[1], m2 = s->m[2];
    ok = ok && salloc(s, &s->x0, 2 * m0 * 16) && salloc(s, &s->a1, 2 * m0 * 32) && salloc(s, &s->p1, 2 * m1 * 32) &&
         salloc(s, &s->a2, 2 * m1 * 64) && salloc(s, &s->p2, 2 * m2 * 64) && salloc(s, &s->a3, 2 * m2 * 128) &&
         salloc(s, &s->a4, 2 * m2 * 64) && salloc(s, &s->u2, 2 * m1 * 64) && salloc(s, &s->a5, 2 * m1 * 32) &&
         salloc(s, &s->u1, 2 * m0 * 32) && salloc(s, &s->y, 4 * m0 * 16);
    ok = ok && salloc(s, &s->dy, 2 * m0 * 16) && salloc(s, &s->du1, 2 * m0 * 32) && salloc(s, &s->da5, 2 * m1 * 32) &&
         salloc(s, &s->du2, 2 * m1 * 64) && salloc(s, &s->da4, 2 * m2 * 64) && salloc(s, &s->da3, 2 * m2 * 128) &&
         salloc(s, &s->dp2, 2 * m2 * 64) && salloc(s, &s->da2, 2 * m1 * 64) && salloc(s, &s->dp1, 2 * m1 * 32) &&
         salloc(s, &s->da1, 2 * m0 * 32);
    ok = ok && salloc(s, &s->scratch, (size_t)scratch);
    s->scratch_bytes = scratch;
    ok = ok && salloc(s, &s->fT, 4 * m0) && salloc(s, &s->fC, 4 * m0) && salloc(s, &s->fqT, 4 * m0) &&
         salloc(s, &s->fqC, 4 * m0) && salloc(s, &s->gT, 4 * m0) && salloc(s, &s->gC, 4 * m0) &&
         salloc(s, &s->tmpA, 4 * m0) && salloc(s, &s->tmpB, 4 * m0) && salloc(s, &s->f1T, 4 * m0) &&
         salloc(s, &s->f1C, 4 * m0) && salloc(s, &s->refT, 4 * m0) && salloc(s, &s->refC, 4 * m0) &&
         salloc(s, &s->part, 4 * 1024) && salloc(s, &s->loss_dev, 4) && salloc(s, &s->cmp_part, 8 * 2 * 4096) &&
         salloc(s, &s->cmp_max, 4) && salloc(s, &s->err, 4);
    if (!ok) { agb_surrogate_destroy(s); return AGB_OUT_OF_MEMORY; }
    cudaMemset(s->err, 0, 4);
    refresh_bf16(s, nullptr);
    if (cudaDeviceSynchronize() != cudaSuccess) { agb_surrogate_destroy(s); return AGB_CUDA_ERROR; }
    *out = s;
    return AGB_OK;
}

agb_status agb_surrogate_window(agb_surrogate* s, uint64_t index, float* T, float* C, float* qT, float* qC,
                                agb_stream stream) {
    if (!s || !T || !C || !qT || !qC) return AGB_INVALID_ARGUMENT;
    make_window(s, index, T, C, qT, qC, reinterpret_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_surrogate_reference(agb_surrogate* s, float* T, float* C, const float* qT, const float* qC,
                                   agb_stream stream) {
    if (!s || !T || !C) return AGB_INVALID_ARGUMENT;
    ftcs_window(s, T, C, qT, qC, reinterpret_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_surrogate_train(agb_surrogate* s, int32_t windows, float* losses, agb_stream stream) {
    if (!s || windows < 0) return AGB_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (int32_t k = 0; k < windows; ++k) {
        make_window(s, (uint64_t)s->adam_t, s->fT, s->fC, s->fqT, s->fqC, st);
        cudaMemcpyAsync(s->gT, s->fT, 4 * (size_t)s->m[0], cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(s->gC, s->fC, 4 * (size_t)s->m[0], cudaMemcpyDeviceToDevice, st);
        ftcs_window(s, s->gT, s->gC, s->fqT, s->fqC, st);
        if (!grad_pass(s, s->fT, s->fC, s->fqT, s->fqC, s->gT, s->gC, st) || !step_adam(s, st))
            return AGB_CUDA_ERROR;
        if (losses) cudaMemcpyAsync(losses + k, s->loss_dev, 4, cudaMemcpyDeviceToHost, st);
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return AGB_CUDA_ERROR;
    uint32_t e = 0;
    cudaMemcpy(&e, s->err, 4, cudaMemcpyDeviceToHost);
    if (losses && windows > 0) s->rep.last_loss = losses[windows - 1];
    return e ? AGB_DEVICE_TIMEOUT : AGB_OK;
}

agb_status agb_surrogate_train_on(agb_surrogate* s, const float* T0, const float* C0, const float* qT,
                                  const float* qC, float* loss, agb_stream stream) {
    if (!s || !T0 || !C0) return AGB_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t b = 4 * (size_t)s->m[0];
    cudaMemcpyAsync(s->fT, T0, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->fC, C0, b, cudaMemcpyDeviceToDevice, st);
    if (qT) cudaMemcpyAsync(s->fqT, qT, b, cudaMemcpyDeviceToDevice, st);
    else cudaMemsetAsync(s->fqT, 0, b, st);
    if (qC) cudaMemcpyAsync(s->fqC, qC, b, cudaMemcpyDeviceToDevice, st);
    else cudaMemsetAsync(s->fqC, 0, b, st);
    cudaMemcpyAsync(s->gT, T0, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->gC, C0, b, cudaMemcpyDeviceToDevice, st);
    ftcs_window(s, s->gT, s->gC, s->fqT, s->fqC, st);
    if (!grad_pass(s, s->fT, s->fC, s->fqT, s->fqC, s->gT, s->gC, st) || !step_adam(s, st)) return AGB_CUDA_ERROR;
    if (loss) {
        cudaMemcpyAsync(loss, s->loss_dev, 4, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return AGB_CUDA_ERROR;
        s->rep.last_loss = *loss;
    }
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_surrogate_gradients(agb_surrogate* s, const float* T0, const float* C0, const float* qT,
                                   const float* qC, const float* T1, const float* C1, float* grads, int64_t cap,
                                   float* loss, agb_stream stream) {
    if (!s || !T0 || !C0 || !T1 || !C1) return AGB_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!grad_pass(s, T0, C0, qT, qC, T1, C1, st)) return AGB_CUDA_ERROR;
    if (grads) {
        if (cap < param_count(s)) return AGB_CAPACITY_EXCEEDED;
        float* p = grads;
        for (Layer& l : s->L) {
            const int64_t n = 27LL * l.cout * l.cin;
            cudaMemcpyAsync(p, l.gw, 4 * n, cudaMemcpyDeviceToHost, st);
            p += n;
            cudaMemcpyAsync(p, l.gb, 4 * l.cout, cudaMemcpyDeviceToHost, st);
            p += l.cout;
        }
    }
    if (loss) cudaMemcpyAsync(loss, s->loss_dev, 4, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return AGB_CUDA_ERROR;
    uint32_t e = 0;
    cudaMemcpy(&e, s->err, 4, cudaMemcpyDeviceToHost);
    return e ? AGB_DEVICE_TIMEOUT : AGB_OK;
}

agb_status agb_surrogate_params(agb_surrogate* s, float* out, int64_t cap, int64_t* count) {
    if (!s || !count) return AGB_INVALID_ARGUMENT;
    *count = param_count(s);
    if (!out) return AGB_OK;
    if (cap < *count) return AGB_CAPACITY_EXCEEDED;
    float* p = out;
    for (Layer& l : s->L) {
        const int64_t n = 27LL * l.cout * l.cin;
        if (cudaMemcpy(p, l.w32, 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return AGB_CUDA_ERROR;
        p += n;
        if (cudaMemcpy(p, l.b32, 4 * l.cout, cudaMemcpyDeviceToHost) != cudaSuccess) return AGB_CUDA_ERROR;
        p += l.cout;
    }
    return AGB_OK;
}

agb_status agb_surrogate_set_params(agb_surrogate* s, const float* in, int64_t count) {
    if (!s || !in || count != param_count(s)) return AGB_INVALID_ARGUMENT;
    const float* p = in;
    for (Layer& l : s->L) {
        const int64_t n = 27LL * l.cout * l.cin;
        if (cudaMemcpy(l.w32, p, 4 * n, cudaMemcpyHostToDevice) != cudaSuccess) return AGB_CUDA_ERROR;
        p += n;
        if (cudaMemcpy(l.b32, p, 4 * l.cout, cudaMemcpyHostToDevice) != cudaSuccess) return AGB_CUDA_ERROR;
        p += l.cout;
    }
    refresh_bf16(s, nullptr);
    return cudaDeviceSynchronize() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_surrogate_advance(agb_surrogate* s, float* T, float* C, const float* qT, const float* qC,
                                 int32_t judge, agb_surrogate_report* rep, agb_stream stream) {
    if (!s || !T || !C) return AGB_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t m = s->m[0];
    ++s->rep.calls;
    const bool do_judge = judge > 0 || (judge == 0 && s->rep.calls % s->d.judge_every == 0);
    if (do_judge) {
        cudaMemcpyAsync(s->refT, T, 4 * (size_t)m, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(s->refC, C, 4 * (size_t)m, cudaMemcpyDeviceToDevice, st);
        ftcs_window(s, s->refT, s->refC, qT, qC, st);
    }
    if (!forward(s, T, C, qT, qC, st)) return AGB_CUDA_ERROR;
    apply_kernel<<<blocks_for(m), 256, 0, st>>>(s->y, T, C, m, s->nm.dt_scale, s->nm.dc_scale);
    s->rep.last_used_surrogate = 1;
    if (do_judge) {
        ++s->rep.judged;
        double res[2][3];
        for (int f = 0; f < 2; ++f) {
            cudaMemsetAsync(s->cmp_max, 0, 4, st);
            const unsigned nb = 1024;
            compare_kernel<<<nb, 256, 0, st>>>(f == 0 ? T : C, f == 0 ? s->refT : s->refC, m, s->cmp_max, s->cmp_part);
            unsigned int mx = 0;
            std::vector<double> part(2 * nb);
            cudaMemcpyAsync(&mx, s->cmp_max, 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(part.data(), s->cmp_part, 8 * 2 * nb, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return AGB_CUDA_ERROR;
            float fm;
            std::memcpy(&fm, &mx, 4);
            double dsum = 0.0, tsum = 0.0;
            for (unsigned b = 0; b < nb; ++b) { dsum += part[2 * b]; tsum += part[2 * b + 1]; }
            res[f][0] = fm; res[f][1] = dsum; res[f][2] = tsum;
        }
        s->rep.last_err_temperature = res[0][0];
        s->rep.last_err_co2 = res[1][0];
        s->rep.last_energy_drift = res[0][2] != 0.0 ? std::fabs(res[0][1] / res[0][2]) : std::fabs(res[0][1]);
        if (!(s->rep.last_err_temperature <= s->d.tol_temperature) || !(s->rep.last_energy_drift <= s->d.tol_energy)) {
            ++s->rep.fallbacks;                           // the judge's FTCS result takes over
            cudaMemcpyAsync(T, s->refT, 4 * (size_t)m, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(C, s->refC, 4 * (size_t)m, cudaMemcpyDeviceToDevice, st);
            s->rep.last_used_surrogate = 0;
        }
    }
    if (rep) *rep = s->rep;
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_surrogate_get_report(agb_surrogate* s, agb_surrogate_report* rep) {
    if (!s || !rep) return AGB_INVALID_ARGUMENT;
    *rep = s->rep;
    return AGB_OK;
}

agb_status agb_surrogate_error_word(agb_surrogate* s, uint32_t* word) {
    if (!s || !word) return AGB_INVALID_ARGUMENT;
    return cudaMemcpy(word, s->err, 4, cudaMemcpyDeviceToHost) == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

}  // extern "C"
