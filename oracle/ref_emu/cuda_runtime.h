// oracle/ref_emu/cuda_runtime.h -- host stand-in for the CUDA runtime calls
// the reference's physics sources make. Device memory is host memory; every
// call is synchronous. TEST INFRASTRUCTURE ONLY (see emu.h).
#pragma once
#include <cstdlib>
#include <cstring>

#include "emu.h"

enum cudaError_t { cudaSuccess = 0, cudaErrorMemoryAllocation = 2, cudaErrorInvalidValue = 1 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3, cudaMemcpyDefault = 4
};
typedef struct emu_stream* cudaStream_t;

namespace emu {
size_t live_allocations();
void* alloc(size_t bytes);
void release(void* p);
}  // namespace emu

template <typename T>
inline cudaError_t cudaMalloc(T** p, size_t bytes) {
    void* q = ::emu::alloc(bytes);
    *p = static_cast<T*>(q);
    return q ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void* p) { ::emu::release(p); return cudaSuccess; }
inline cudaError_t cudaMemset(void* p, int v, size_t bytes) { std::memset(p, v, bytes); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t bytes, cudaMemcpyKind) {
    std::memmove(d, s, bytes); return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "emulated error"; }
