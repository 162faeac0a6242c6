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
    double* co2_want;        // per slot: the uptake the demand pass computed (the uptake pass reads it back)
    int32_t* co2_vox;        // per slot: its CO2 voxel as the demand pass found it, -1 for a cell that booked no
                             // demand (the uptake pass and the CO2 flush read it back); null: recompute
};

// ---------------------------------------------------------------------------
// Batched stages (agb_batch): one launch runs a stage for many chambers. The
// grid's blocks are shared out over the chambers: block k works for chamber
// map[k] >> 16 as its block map[k] & 0xFFFF of that chamber's nblk, with the
// chamber's entry of a device table of ChamberArgs, through the same kernel
// bodies as the per-world launches.
// ---------------------------------------------------------------------------
struct ChamberArgs {
    DevState* S;
    Ctx c;                        // the chamber's context as this stage sees it
    TickParams p;
    GridDev g;                    // flush: the grid flushed; integrate: the diffused CO2 grid
    int32_t* stamp_idx;
    double* factor;
    float *fx, *fy, *fz;
    unsigned long long* demand;   // CO2 rationing words (null: no CO2 grid)
    LifeBuffers life;
    uint32_t *kalt, *valt, *hist; // hash sort scratch
    double gv;
    int32_t nblk;                 // the chamber's blocks in this launch
    int32_t arg;                  // stage switch (cell step: feed | taxis << 1; divide: compaction allowed)
    int32_t passes, max_tiles;    // hash sort: digit passes, tiles per pass
    int32_t radix_bits;           // hash sort: bits per digit (8 or 9)
};

// A batched kernel NAME(tab, map): finds its chamber and block, then CALL
// (which sees the chamber's arguments as `a` and its block as `blk`).
#define AGB_BATCHED(NAME, THREADS, CALL) AGB_BATCHED_MB(NAME, THREADS, 1, CALL)
// ... with at least MINB resident blocks per SM (a register budget).
#define AGB_BATCHED_MB(NAME, THREADS, MINB, CALL)                                                    \
    __global__ void __launch_bounds__(THREADS, MINB) NAME(const ChamberArgs* __restrict__ tab,        \
                                                          const uint32_t* __restrict__ map) {        \
        pdl_wait();                                                                                  \
        int32_t ch_, x_;                                                                             \
        batch_block(map, ch_, x_);                                                                   \
        const ChamberArgs& a = tab[ch_];                                                             \
        const Blk blk{x_, a.nblk};                                                                   \
        CALL;                                                                                        \
    }

enum class BStage : int32_t {
    Thermal, ClearStamps, Stamp, Occlusion, SweepRows, SweepLines, CellStep, Integrate,   // k_cells.cu
    Flush,                                                                                // k_grid.cu
    HashClear, KeyHist, Radix4, Radix4x9, Radix8, Ranges,                                 // k_hash.cu
    UptakeMark, Scan, Divide, Keep, ScatterSrc, Gather, Swap                              // k_life.cu
};
// Threads per block of a batched stage.
int32_t bstage_threads(BStage st);
// Enqueue one batched stage over `blocks` blocks. `arg`: the radix pass index
// (Radix4/8) or the scan gate (Scan: 0 division, 1 compaction).
void launch_batched(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                    cudaStream_t s);
// The per-file halves of launch_batched; each returns false for a stage it does not own.
bool launch_batched_cells(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, cudaStream_t s);
bool launch_batched_grid(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, cudaStream_t s);
bool launch_batched_hash(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                         cudaStream_t s);
bool launch_batched_life(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                         cudaStream_t s);
// Blocks of a chamber in a batched stage, as the per-world launches size them.
int32_t hash_clear_blocks(int32_t passes, int32_t max_tiles, int32_t radix_bits);
int32_t scan_blocks(int32_t capacity);
// Blocks of the x-axis sweep over `lines` rows: a warp per 32 rows, 8 warps a block.
inline int32_t sweep_rows_blocks(int64_t lines) {
    const int64_t b = ((lines + 31) / 32 + 7) / 8;
    return (int32_t)(b < 65535 ? b : 65535);
}
// Digit passes, tiles per pass and digit width of the hash sort for a world,
// and whether its tiles are 1024 keys (Radix4, Radix4x9 for 9-bit digits) or
// 2048 (Radix8).
void hash_sort_shape(const HashDev& h, int32_t capacity, int32_t& passes, int32_t& max_tiles, bool& per4,
                     int32_t& radix_bits);

// co2_uptake_rate (src/sim/lifecycle.cuh:24-28): FP64 in the reference's
// operation order. The rationing below compares a voxel's booked demand with
// its contents, and only the reference's precision keeps the total taken
// within what the voxel holds (in FP32 the relative error of ~1e-7 let a
// drained voxel go slightly negative).
__device__ __forceinline__ double co2_uptake_rate_d(double c) {
    if (c <= 0.0) return 0.0;
    return __ddiv_rn(__dmul_rn(AGB_LIFE_CO2_UPTAKE_MAX, c), __dadd_rn(c, AGB_LIFE_CO2_HALF_SATURATION));
}

// fixed_atomic.cuh to_fixed: llround(value * scale).
__device__ __forceinline__ long long to_fixed_d(double v, double scale) {
    return llround(__dmul_rn(v, scale));
}

// One live cell's CO2 demand at (x, y, z) into the voxel's rationing word, as
// a concentration (demand_kernel body, src/sim/lifecycle.cu:41-57); gv is the
// voxel volume. The cell's wanted uptake is kept in want[i]: the uptake pass
// (uptake_kernel, lifecycle.cu:62-86) evaluates the same expression on the
// same voxel value, so it reads it back instead of dividing again.
__device__ __forceinline__ void co2_demand_cell(const GridDev& C2, const TickParams& p, float x, float y, float z,
                                                unsigned long long* demand, double gv, double* want_out,
                                                int32_t* vox_out, int32_t i) {
    const int64_t idx = grid_nearest(C2, x, y, z);
    const double want = __dmul_rn(co2_uptake_rate_d((double)C2.value[idx]), p.dt_bio);
    want_out[i] = want;
    if (vox_out) vox_out[i] = (int32_t)idx;
    if (want > 0.0) deposit_fixed(&demand[idx], to_fixed_d(div_known(want, gv, C2.vol_inv), C2.scale));
}

// `first`: the tick's first thermal substep (it records each cell's voxel in c.t_vox).
void launch_thermal(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, bool first, cudaStream_t s);
// flash_step (src/sim/flash.cu:59-67) while the spin-drive flash is armed.
void launch_flash(DevState* S, double dt, double power, unsigned long long* accum, int32_t blocks, cudaStream_t s);
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
// The two halves of launch_motion: forces (field sample + contact walk) and
// integration. With `demand` set, integration also enters each live cell's
// CO2 demand at its new position into `demand` from the grid `co2` (the
// lifecycle's first pass, which needs the CO2 as diffused this tick).
void launch_forces(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                   int32_t blocks, int lanes, cudaStream_t s);
void launch_integrate(DevState* S, const Ctx& c, const TickParams& p, const float* fx, const float* fy,
                      const float* fz, int32_t blocks, const GridDev& co2, unsigned long long* demand,
                      double gv, double* want, int32_t* vox, cudaStream_t s);
// Feeding (when `feed`), taxis (when `taxis`) and forces in one per-cell pass
// with one neighbour walk: the same cell values as launch_feed, launch_taxis
// and launch_forces in turn, with two kernels fewer on the tick's critical
// path (integration follows separately).
// `c` is the motion context (CO2/N2 as they stood before this tick's slow
// fields; feeding reads only the irradiance grid).
void launch_cell_step(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                      int32_t blocks, int lanes, bool feed, bool taxis, cudaStream_t s);
// lifecycle_step (src/sim/lifecycle.cu:208-294), compaction included.
// `demand_done`: integration already entered this tick's CO2 demand.
void launch_lifecycle(DevState* S, const Ctx& c, const TickParams& p, const LifeBuffers& b,
                      bool compaction_allowed, int32_t blocks, cudaStream_t s, bool demand_done = false);
// cell_store_compact (src/sim/cell_store.cu:414-456) on its own.
void launch_compact(DevState* S, const Ctx& c, const LifeBuffers& b, int32_t blocks, cudaStream_t s);
// stats_step (src/sim/stats.cu:79-100): fixed-point sums into acc[12].
void launch_stats(DevState* S, const Ctx& c, unsigned long long* acc, int32_t blocks, cudaStream_t s);
// spawn_kernel (src/sim/cell_store.cu:42-130) for `count` new cells.
void launch_spawn(DevState* S, const Ctx& c, const agb_spawn& p, int32_t blocks, cudaStream_t s);
// Every occupied slot's energy set to `energy` (cell_store.cu:281-297).
void launch_set_charge(DevState* S, double energy, int32_t blocks, cudaStream_t s);

// ---------------------------------------------------------------------------
// Taumoeba, the predator (src/sim/predation.cuh:82-118, k_tau.cu)
// ---------------------------------------------------------------------------
struct TauSoA {
    uint64_t* id;
    uint32_t* flags;
    double *x, *y, *z, *vx, *vy, *vz;
    float *dir_x, *dir_y, *dir_z;
    double *biomass, *prey_biomass;
    float *digest_timer, *tolerance;
    uint32_t* generation;
    uint64_t* rng_state;
    float *density_ema, *run_timer;
    int32_t* target;
};
// Device-resident store state: the live and spare arrays (compaction writes
// the spare and swaps), the count and the next predator id.
struct TauState {
    TauSoA cur, spare;
    int32_t count, capacity;
    uint64_t next_id;
};
// Per-world constants of a predator tick, computed on the host in FP64 with
// the reference's expressions: the OU step of TAU_MASS under the Stokes drag
// at the ambient temperature (ou_coefficients, integrator.cuh:103-121), the
// run-and-tumble memory weight (predation.cuh:38), the walls.
struct TauParams {
    double dt, dt_bio, alpha;
    float dt_f, dt_bio_f;
    double gamma, ome, inv_beta, s_rr, s_vv, noise_a, noise_b;
    double lo[3], hi[3], half[3], span[3];
    int32_t boundary_x, boundary_y, noise, disposition, compaction;
};
// The 20 arrays carved from one blob of `capacity` predators (snapshot order).
TauSoA tau_carve(void* blob, int32_t capacity);
size_t tau_blob_bytes(int32_t capacity);
// taumoeba_spawn (predation.cu:33-74, 420-432): `count` predators appended at
// the device-side count.
void launch_tau_spawn(TauState* T, int32_t count, uint64_t seed, const TauParams& p, cudaStream_t s);
// predation_step (predation.cu:434-484): claim reset, hunt, resolve, nitrogen,
// then division and (if enabled) compaction in one CTA.
void launch_predation(TauState* T, DevState* S, const HashDev& h, const GridDev& n2, const TauParams& p,
                      unsigned long long* claim, int32_t cell_capacity, int32_t tau_capacity, cudaStream_t s);
// stats_taumoeba_kernel (stats.cu:65-73): alive count into acc[11], tolerance into acc[6].
void launch_tau_stats(TauState* T, int32_t tau_capacity, unsigned long long* acc, cudaStream_t s);

}  // namespace agb
