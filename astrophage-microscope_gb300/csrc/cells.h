// cells.h -- launchers of the per-cell stage kernels (k_cells.cu, k_life.cu).
#pragma once

#include "kernels.h"
#include "world.cuh"

namespace agb {

// Scratch the lifecycle and compaction passes share (sized at capacity).
struct LifeBuffers {
    int32_t* flags;          // 0/1 predicate per slot (divides, or survives compaction)
    int32_t* prefix;         // exclusive prefix of `flags`
    int32_t* tile_sums;      // per-tile totals for the two-level scan
    int32_t* src;            // compaction: source slot of each output slot
    unsigned long long* co2_demand;   // per CO2 voxel, fixed point (src/sim/world.cuh:108)
};

void launch_thermal(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, cudaStream_t s);
// `lanes` (1, 2, 4 or 8) threads share each cell's neighbour walk in the
// feeding and contact-force kernels; `blocks` sizes one thread per cell.
void launch_emission(DevState* S, const Ctx& c, const TickParams& p, int32_t* stamp_idx, double* factor,
                     bool stamp, int32_t blocks, int lanes, cudaStream_t s);
// The two halves of launch_emission: the irradiance field (stamps, occlusion
// factors, sweep; needs the post-thermal cells, not the hash) and feeding
// (walks the hash).
void launch_emission_prep(DevState* S, const Ctx& c, const TickParams& p, int32_t* stamp_idx, double* factor,
                          bool stamp, int32_t blocks, cudaStream_t s);
void launch_feed(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, int lanes, cudaStream_t s);
// taxis_step (src/sim/taxis.cu:13-85): run-and-tumble state machine, emission.
void launch_taxis(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, cudaStream_t s);
void launch_motion(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                   int32_t blocks, int lanes, cudaStream_t s);
// Feeding (when `feed`), taxis (when `taxis`) and motion in one per-cell pass
// plus integration: the same cell values as launch_feed, launch_taxis and
// launch_motion in turn, with two kernels fewer on the tick's critical path.
// `c` is the motion context (CO2/N2 as they stood before this tick's slow
// fields; feeding reads only the irradiance grid).
void launch_cell_step(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                      int32_t blocks, int lanes, bool feed, bool taxis, cudaStream_t s);
// lifecycle_step (src/sim/lifecycle.cu:208-294), compaction included.
void launch_lifecycle(DevState* S, const Ctx& c, const TickParams& p, const LifeBuffers& b,
                      bool compaction_allowed, int32_t blocks, cudaStream_t s);
// cell_store_compact (src/sim/cell_store.cu:414-456) on its own.
void launch_compact(DevState* S, const Ctx& c, const LifeBuffers& b, int32_t blocks, cudaStream_t s);
// stats_step (src/sim/stats.cu:79-100): fixed-point sums into acc[12].
void launch_stats(DevState* S, const Ctx& c, unsigned long long* acc, int32_t blocks, cudaStream_t s);
// spawn_kernel (src/sim/cell_store.cu:42-130) for `count` new cells.
void launch_spawn(DevState* S, const Ctx& c, const agb_spawn& p, int32_t blocks, cudaStream_t s);

}  // namespace agb
