// noalloc.cu -- diffusion of a caller-owned field without any device allocation.
//
// Who needs this: code that owns one field buffer but may not allocate device
// memory -- a host application with a fixed, pre-reserved memory budget (a
// render or physics engine that forbids allocation after start-up), a plugin
// running inside a host that owns the CUDA context and its allocator policy,
// or a real-time loop where cudaMalloc's implicit device synchronisation would
// stall the frame. grid_diffuse needs a second buffer of the field's size to
// ping-pong against; here that buffer is a fixed array compiled into the
// library instead of something the caller allocates.
//
// The array holds AGB_NOALLOC_MAX_VOXELS floats (16 MiB) on every GPU that
// loads the library, for the life of the process. All calls share it, so calls
// whose work overlaps on the GPU (different streams, or different host threads
// on one device) race on it; serialise them. Nothing in it has to start at zero:
// every pass writes each voxel of its destination before any voxel is read.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "kernels.h"

namespace {

__device__ __align__(256) float g_noalloc_scratch[AGB_NOALLOC_MAX_VOXELS];

constexpr int kMaxDevices = 64;
float* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// The array's device address on the current device. Host code only sees a
// host-side stand-in for a __device__ symbol, so the real address is asked
// from the runtime once per device (with that device current) and kept.
agb_status scratch_on_current_device(float** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AGB_CUDA_ERROR;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return AGB_CUDA_ERROR;
        g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[dev];
    return AGB_OK;
}

}  // namespace

extern "C" agb_status agb_grid_diffuse_noalloc(float* value, int32_t nx, int32_t ny, int32_t nz, double dx,
                                               double diffusivity, double dt, const int32_t bc[6],
                                               const double face_value[6], agb_stream stream) {
    if (value == nullptr || bc == nullptr || face_value == nullptr || nx < 2 || ny < 2 || nz < 1 ||
        !(dx > 0.0) || !(diffusivity > 0.0) || !(dt >= 0.0))
        return AGB_INVALID_ARGUMENT;
    const int64_t count = (int64_t)nx * ny * nz;
    if (count > (int64_t)AGB_NOALLOC_MAX_VOXELS) return AGB_CAPACITY_EXCEEDED;
    // Within the voxel limit, a very tall and thin grid (e.g. 4 x 1,048,576 x 1)
    // still exceeds the stencil's launch grid (65,535 blocks of 8 rows along y,
    // and of 8 planes along z): refused before anything is launched or copied.
    if (!agb::ftcs_plain_fits(nx, ny, nz)) return AGB_UNSUPPORTED;
    // Substeps and coefficient as grid_diffuse computes them (1/6 bound in 3-D).
    const double lim = nz > 1 ? 6.0 : 4.0;
    const int32_t steps = (int32_t)(dt / (dx * dx / (lim * diffusivity))) + 1;
    if (steps <= 0) return AGB_OK;
    const float coeff = (float)(diffusivity * (dt / steps) / (dx * dx));
    if (!(nz > 1 ? coeff <= (float)(1.0 / 6.0) : coeff <= 0.25f)) return AGB_INVALID_ARGUMENT;
    float* scratch = nullptr;
    const agb_status rc = scratch_on_current_device(&scratch);
    if (rc != AGB_OK) return rc;

    agb::GridDev g{};
    g.nx = nx; g.ny = ny; g.nz = nz; g.count = count; g.enabled = 1;
    float face[6];
    for (int k = 0; k < 6; ++k) face[k] = (float)face_value[k];
    const float robin = (float)(dx * AGB_AIR_CONVECTION_H / AGB_WATER_CONDUCTIVITY);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    float* src = value;
    float* dst = scratch;
    for (int32_t k = 0; k < steps; ++k) {
        // A pass that fails to launch ends the call before the final copy, so
        // the caller's buffer is never overwritten from a half-done sequence.
        if (agb::launch_ftcs(g, src, dst, coeff, bc, face, robin, nullptr, nullptr, nullptr, s) != cudaSuccess)
            return AGB_CUDA_ERROR;
        float* t = src; src = dst; dst = t;
    }
    if (src != value &&
        cudaMemcpyAsync(value, src, sizeof(float) * (size_t)count, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return AGB_CUDA_ERROR;
    return AGB_OK;
}
