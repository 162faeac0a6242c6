// nn.h -- building blocks of the learned field surrogate: tensor-core
// convolutions (conv_tc.cu) and the memory-bound layers around them
// (nn_ops.cu). Activations are channels-last BF16 [D][H][W][C]; weights are
// [27][Cout][Cin] BF16 (tap t = (dz+1)*9 + (dy+1)*3 + (dx+1)).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace agb {
namespace nn {

struct Conv3Args {
    int32_t D, H, W, cin, cout;
    const float* bias;              // [cout] or nullptr
    int32_t act;                    // 0: none, 1: ReLU
    const __nv_bfloat16* mask;      // [M][cout] or nullptr: output zeroed where mask <= 0
    void* out;                      // [M][cout], BF16 or FP32
    int32_t out_f32;
    uint32_t* err;                  // device error word (bounded wait expired)
};

struct WgradArgs {
    int32_t D, H, W, cin, cout;
    int32_t splits, rows_per_split; // voxel rows (z, y) per CTA
    float* partial;                 // [27][splits][cout][cin]
    uint32_t* err;
};

// Shapes the tensor-core kernels take: W in {32, 64} or a multiple of 128 up
// to 256, H*W a multiple of 128; cin 16, 32 or a multiple of 64 (<= 256),
// cout 16/32/64/128 (forward). Weight gradient: W 32 or a multiple of 64,
// cin 16/32/64/128, cout <= 128.
bool conv3_supported(int D, int H, int W, int cin, int cout);
bool wgrad_supported(int D, int H, int W, int cin, int cout);
cudaError_t conv3(const Conv3Args& a, const void* x, const void* w, cudaStream_t s);
// dyt: [cout][M] BF16; xt3: [3][cin][M] BF16 (x shifted by -1, 0, +1).
cudaError_t wgrad(const WgradArgs& a, const void* dyt, const void* xt3, cudaStream_t s);

// nn_ops.cu
void to_channel_major(const __nv_bfloat16* x, __nv_bfloat16* xt, int64_t m, int c, cudaStream_t s);
void to_channel_major_shifted(const __nv_bfloat16* x, __nv_bfloat16* xt3, int D, int H, int W, int c,
                              cudaStream_t s);
void reduce_partials(const float* partial, float* dw, int splits, int64_t per_tap, float scale, int accumulate,
                     cudaStream_t s);
void bias_grad(const __nv_bfloat16* dy, float* db, int64_t m, int c, float* scratch, cudaStream_t s);
void flip_weights(const __nv_bfloat16* w, __nv_bfloat16* wf, int cout, int cin, cudaStream_t s);
void avgpool2(const __nv_bfloat16* x, __nv_bfloat16* y, int D, int H, int W, int c, cudaStream_t s);
void avgpool2_backward_add(const __nv_bfloat16* dy, const __nv_bfloat16* dskip, const __nv_bfloat16* act,
                           __nv_bfloat16* dx, int D, int H, int W, int c, cudaStream_t s);
void upsample2_add(const __nv_bfloat16* coarse, const __nv_bfloat16* skip, __nv_bfloat16* y, int D, int H, int W,
                   int c, cudaStream_t s);
void upsample2_backward(const __nv_bfloat16* dy, const __nv_bfloat16* act, __nv_bfloat16* dcoarse, int D, int H,
                        int W, int c, cudaStream_t s);

}  // namespace nn
}  // namespace agb
