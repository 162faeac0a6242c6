// nn_abi.cu -- C entry points of the surrogate's layer primitives (tensor-core
// convolution, weight gradient, weight flip) on caller-owned device buffers.
// They have no counterpart in the reference; they exist so the layers can be
// checked one by one against a CPU restatement.
#include <cuda_runtime.h>

#include "../../include/agb.h"
#include "nn.h"

namespace {

int wgrad_splits(int rows) {
    static int sms = 0;
    if (sms == 0) {
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
        if (sms <= 0) sms = 1;
    }
    int s = (4 * sms + 26) / 27;
    if (s > rows) s = rows;
    return s < 1 ? 1 : s;
}

size_t al(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace

extern "C" {

agb_status agb_nn_conv3(const void* x, const void* w, const float* bias, int32_t D, int32_t H, int32_t W,
                        int32_t cin, int32_t cout, int32_t act, const void* mask, void* out, int32_t out_f32,
                        uint32_t* err, agb_stream s) {
    if (!x || !w || !out || !err || !agb::nn::conv3_supported(D, H, W, cin, cout)) return AGB_INVALID_ARGUMENT;
    agb::nn::Conv3Args a{D, H, W, cin, cout, bias, act, static_cast<const __nv_bfloat16*>(mask), out, out_f32, err};
    return agb::nn::conv3(a, x, w, reinterpret_cast<cudaStream_t>(s)) == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

int64_t agb_nn_wgrad_scratch_bytes(int32_t D, int32_t H, int32_t W, int32_t cin, int32_t cout) {
    const int64_t m = (int64_t)D * H * W;
    const int splits = wgrad_splits(D * H);
    return (int64_t)(al(2 * (size_t)cout * m) + al(2 * 3 * (size_t)cin * m) +
                     al(4 * 27 * (size_t)splits * cout * cin) + al(4 * 1024 * (size_t)(cout > 0 ? cout : 1)));
}

agb_status agb_nn_wgrad(const void* x, const void* dy, int32_t D, int32_t H, int32_t W, int32_t cin, int32_t cout,
                        float* dw, float* db, void* scratch, int64_t scratch_bytes, uint32_t* err, agb_stream stream) {
    if (!x || !dy || !dw || !scratch || !err || !agb::nn::wgrad_supported(D, H, W, cin, cout))
        return AGB_INVALID_ARGUMENT;
    if (scratch_bytes < agb_nn_wgrad_scratch_bytes(D, H, W, cin, cout)) return AGB_CAPACITY_EXCEEDED;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t m = (int64_t)D * H * W;
    const int rows = D * H;
    const int splits = wgrad_splits(rows);
    char* p = static_cast<char*>(scratch);
    auto* dyt = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(2 * (size_t)cout * m);
    auto* xt3 = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(2 * 3 * (size_t)cin * m);
    auto* partial = reinterpret_cast<float*>(p);
    p += al(4 * 27 * (size_t)splits * cout * cin);
    auto* colsum = reinterpret_cast<float*>(p);
    const auto* xb = static_cast<const __nv_bfloat16*>(x);
    const auto* dyb = static_cast<const __nv_bfloat16*>(dy);
    agb::nn::to_channel_major(dyb, dyt, m, cout, s);
    agb::nn::to_channel_major_shifted(xb, xt3, D, H, W, cin, s);
    agb::nn::WgradArgs a{D, H, W, cin, cout, splits, (rows + splits - 1) / splits, partial, err};
    if (agb::nn::wgrad(a, dyt, xt3, s) != cudaSuccess) return AGB_CUDA_ERROR;
    agb::nn::reduce_partials(partial, dw, splits, (int64_t)cout * cin, 1.0f, 0, s);
    if (db) agb::nn::bias_grad(dyb, db, m, cout, colsum, s);
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

agb_status agb_nn_flip_weights(const void* w, void* wf, int32_t cout, int32_t cin, agb_stream s) {
    if (!w || !wf || cout <= 0 || cin <= 0) return AGB_INVALID_ARGUMENT;
    agb::nn::flip_weights(static_cast<const __nv_bfloat16*>(w), static_cast<__nv_bfloat16*>(wf), cout, cin,
                          reinterpret_cast<cudaStream_t>(s));
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA_ERROR;
}

}  // extern "C"
