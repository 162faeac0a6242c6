// oracle/ref_emu/emu.h -- serial host emulation of the small CUDA subset the
// reference's per-tick physics uses, so its own src/sim + src/fields sources
// compile with g++ and run on the CPU as the parity oracle.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product links this.
//
// What the reference's kernels need (survey of src/sim/*.cu, src/fields/*.cu):
// 1-D/2-D grids of independent threads, no shared memory, no barriers, no warp
// intrinsics, integer atomics (add/max/min), cudaMalloc/Memset/Memcpy on the
// default stream, and CUB's stable radix sort and exclusive scan (cub shim).
// Because no kernel communicates between threads except through integer
// atomics, running every thread to completion in (block, thread) order is a
// legal schedule and yields the reference's results.
//
// Kernel launches `k<<<g, b>>>(args)` are rewritten by the build recipe to
// `EMU_LAUNCH((g, b), k)(args)`; everything else is the reference verbatim.
#pragma once

#ifndef __CUDACC__
#define __CUDACC__ 1   // the reference gates its device-side deposits on this
#endif
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

#include <cstddef>
#include <cstdint>

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int x_ = 1, unsigned int y_ = 1, unsigned int z_ = 1) : x(x_), y(y_), z(z_) {}
};

namespace emu {
extern uint3 g_block_idx, g_thread_idx;
extern dim3 g_block_dim, g_grid_dim;
}  // namespace emu

#define blockIdx  (::emu::g_block_idx)
#define threadIdx (::emu::g_thread_idx)
#define blockDim  (::emu::g_block_dim)
#define gridDim   (::emu::g_grid_dim)

namespace emu {

template <typename F>
struct BoundLaunch {
    dim3 grid, block;
    F fn;
    template <typename... A>
    void operator()(A... args) const {
        const dim3 saved_grid = g_grid_dim, saved_block = g_block_dim;
        g_grid_dim = grid;
        g_block_dim = block;
        for (unsigned bz = 0; bz < grid.z; ++bz)
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; ++bx)
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                g_block_idx = uint3{bx, by, bz};
                                g_thread_idx = uint3{tx, ty, tz};
                                fn(args...);   // by value: each thread gets its own copies
                            }
        g_grid_dim = saved_grid;
        g_block_dim = saved_block;
    }
};

struct Launch {
    dim3 grid, block;
    template <typename F>
    BoundLaunch<F> operator+(F f) const { return BoundLaunch<F>{grid, block, f}; }
};

inline Launch make_launch(dim3 g, dim3 b) { return Launch{g, b}; }
inline Launch make_launch(dim3 g, dim3 b, size_t, void* = nullptr) { return Launch{g, b}; }

}  // namespace emu

#define EMU_LAUNCH(dims, kernel) \
    (::emu::make_launch dims + [&](auto... _emu_args) { kernel(_emu_args...); })

// --- integer atomics (serial: plain read-modify-write) ----------------------
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
    const unsigned long long o = *p; *p = o + v; return o;
}
inline unsigned int atomicAdd(unsigned int* p, unsigned int v) { const unsigned o = *p; *p = o + v; return o; }
inline int atomicAdd(int* p, int v) { const int o = *p; *p = o + v; return o; }
inline unsigned long long atomicMax(unsigned long long* p, unsigned long long v) {
    const unsigned long long o = *p; if (v > o) *p = v; return o;
}
inline unsigned long long atomicMin(unsigned long long* p, unsigned long long v) {
    const unsigned long long o = *p; if (v < o) *p = v; return o;
}
inline unsigned long long atomicExch(unsigned long long* p, unsigned long long v) {
    const unsigned long long o = *p; *p = v; return o;
}
