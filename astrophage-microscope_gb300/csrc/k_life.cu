// k_life.cu -- lifecycle (src/sim/lifecycle.cu:26-294), compaction
// (src/sim/cell_store.cu:368-456), telemetry (src/sim/stats.cu:27-153) and
// the seeded spawn (src/sim/cell_store.cu:42-130).
//
// The reference copies the birth and death counts to the host every tick and
// again inside compaction (lifecycle.cu:250-252, cell_store.cu:428) to decide
// whether to scan, divide and compact. Here those decisions are read from
// device memory by the kernels themselves, so the tick never waits on the host
// and can be captured as a CUDA graph. Slot, id and daughter-stream assignment
// come from the same exclusive prefix sums, so they are identical.
#include <cuda_runtime.h>

#include "cells.h"

namespace agb {

namespace {

constexpr int ST = 256;           // scan threads per block
constexpr int SITEMS = 4;
constexpr int STILE = ST * SITEMS;

// ---------------------------------------------------------------------------
// CO2 uptake (demand_kernel / uptake_kernel, lifecycle.cu:41-86)
// ---------------------------------------------------------------------------
// demand_kernel (lifecycle.cu:41-57). The tick itself folds this pass into
// integration (integrate_kernel), which has the moved cell at hand; the
// per-stage lifecycle runs it here.
__global__ void __launch_bounds__(256) demand_kernel(DevState* S, Ctx c, TickParams p,
                                                     unsigned long long* demand, double gv, double* want,
                                                     int32_t* vox) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->count;
    const GridDev C2 = c.g[AGB_FIELD_CO2];
    AGB_FOR_CELLS(i, n) {
        const uint32_t f = v.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED)) continue;
        if (!(f & AGB_FLAG_ALIVE)) {
            if (vox) vox[i] = -1;
            continue;
        }
        co2_demand_cell(C2, p, d2f(v.x[i]), d2f(v.y[i]), d2f(v.z[i]), demand, gv, want, vox, i);
    }
}

__device__ __forceinline__ bool ready_to_divide(const Ctx& c, const SoA& v, int32_t i) {
    if (c.division_predicate == AGB_DIVIDE_ENERGY) return v.energy[i] >= c.division_energy;
    return v.co2_held[i] >= c.co2_quota;                    // lifecycle.cuh:33-36
}

// Per cell, after every demand is in: CO2 uptake (uptake_kernel,
// lifecycle.cu:59-86; `demand` null when there is no CO2 grid), then
// death_kernel + mark_kernel (lifecycle.cu:90-134). Each reads one cell and
// writes only that cell, besides uptake's deposit into its voxel's deposit
// word, which nothing here reads; the CO2 flush that must follow every
// deposit (lifecycle.cu:235) runs in the divide pass.
__device__ __forceinline__ void uptake_mark_kernel_body(DevState* S, const Ctx& c, const TickParams& p,
                                                        const unsigned long long* __restrict__ demand, double gv,
                                                        const double* __restrict__ want_in,
                                                        const int32_t* __restrict__ vox_in, int32_t* divflag,
                                                        Blk blk) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    const GridDev C2 = c.g[AGB_FIELD_CO2];
    int32_t births = 0, deads = 0;
    AGB_FOR_CELLS_B(i, blk, n) {
        uint32_t f = v.flags[i];
        if (demand && (f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE)) {
            // uptake_kernel (lifecycle.cu:62-86) in FP64, the reference's order.
            const int64_t idx = vox_in ? (int64_t)vox_in[i] : grid_nearest(C2, d2f(v.x[i]), d2f(v.y[i]), d2f(v.z[i]));
            const double available = (double)C2.value[idx];
            const double want = want_in[i];                 // rate(available) * dt, from the demand pass
            if (want > 0.0) {
                const double asked = div_known((double)(long long)demand[idx], C2.scale, C2.scale_inv);  // from_fixed
                double taken = want;
                if (asked > available && asked > 0.0) taken = __dmul_rn(want, __ddiv_rn(available, asked));
                if (taken > 0.0) {
                    v.co2_held[i] = __dadd_rn(v.co2_held[i], taken);
                    deposit_fixed(&C2.deposit[idx], to_fixed_d(div_known(-taken, gv, C2.vol_inv), C2.scale));
                }
            }
        }
        if ((f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE) && v.t_local[i] > c.lethal_f) {
            f &= ~AGB_FLAG_ALIVE;
            v.flags[i] = f;
            v.death_cause[i] = AGB_DEATH_OVERHEATED;
            v.emit_power[i] = 0.0f;
            if (c.store_disposition != AGB_STORE_RETAIN) v.energy[i] = 0.0;   // corpse_energy
        }
        const bool occ = (f & AGB_FLAG_OCCUPIED) != 0u, alive = (f & AGB_FLAG_ALIVE) != 0u;
        const bool div = occ && alive && ready_to_divide(c, v, i);
        divflag[i] = div ? 1 : 0;
        births += div;
        deads += (occ && !alive);
    }
    // Counts are order-free integer sums: one atomic per warp.
    for (int o = 16; o > 0; o >>= 1) {
        births += __shfl_down_sync(0xFFFFFFFFu, births, o);
        deads += __shfl_down_sync(0xFFFFFFFFu, deads, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (births) atomicAdd(&S->births, births);
        if (deads) atomicAdd(&S->deads, deads);
    }
}

__global__ void __launch_bounds__(256) uptake_mark_kernel(DevState* S, Ctx c, TickParams p,
                                                          const unsigned long long* __restrict__ demand,
                                                          double gv, const double* __restrict__ want,
                                                          const int32_t* __restrict__ vox, int32_t* divflag) {
    pdl_wait();
    uptake_mark_kernel_body(S, c, p, demand, gv, want, vox, divflag, grid_blk());
}

// ---------------------------------------------------------------------------
// Two-level exclusive scan of a 0/1 predicate (the reference's CUB
// ExclusiveSum, lifecycle.cu:269-270 and cell_store.cu:422). `gate` selects
// the device flag that says whether a scan is needed this tick.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool scan_gate(const DevState* S, int gate) {
    return gate == 0 ? S->births > 0 : S->compact_now != 0;
}

constexpr uint32_t SCAN_AGG = 1u << 30, SCAN_PRE = 2u << 30, SCAN_VALUE = (1u << 30) - 1u;
constexpr uint32_t SCAN_LOOKBACK_LIMIT = 1u << 24;

// Single pass (decoupled look-back): a CTA takes the next 1024-element tile
// (tiles are numbered in the order CTAs start, so every tile it waits on is
// already running), scans it, publishes its total, takes the exclusive prefix
// of the tiles before it from their published totals/prefixes and writes the
// prefix. The last CTA to finish clears the status words and counters for
// the next scan. gate 1 (compaction) also stores the grand total in S->live.
// Waits are bounded; a timeout sets the error word.
__device__ __forceinline__ void scan_kernel_body(DevState* S, const int32_t* __restrict__ flag, int32_t* prefix,
                                                 uint32_t* status, int gate, Blk blk) {
    if (!scan_gate(S, gate)) return;                     // uniform over the grid
    __shared__ int32_t warp_tot[SITEMS][ST / 32];
    __shared__ uint32_t tile_sh;
    __shared__ int32_t excl_sh;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int32_t n = S->count;
    const int32_t ntiles = (n + STILE - 1) / STILE;
    if (threadIdx.x == 0) tile_sh = atomicAdd(&S->scan_tile, 1u);
    __syncthreads();
    const int32_t tile = (int32_t)tile_sh;
    if (tile < ntiles) {
        const int64_t base = (int64_t)tile * STILE;
        int32_t x[SITEMS], inc[SITEMS];
        for (int u = 0; u < SITEMS; ++u) {
            const int64_t e = base + u * ST + threadIdx.x;
            x[u] = e < n ? flag[e] : 0;
            int32_t v = x[u];
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
                if (lane >= o) v += y;
            }
            inc[u] = v;
            if (lane == 31) warp_tot[u][w] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int32_t agg = 0;
            for (int u = 0; u < SITEMS; ++u)
                for (int q = 0; q < ST / 32; ++q) agg += warp_tot[u][q];
            int32_t excl = 0;
            if (tile == 0) {
                atomicExch(&status[0], SCAN_PRE | (uint32_t)agg);
            } else {
                atomicExch(&status[tile], SCAN_AGG | (uint32_t)agg);
                bool ok = true;
                for (int j = tile - 1; j >= 0;) {
                    uint32_t vj = 0, it = 0;
                    for (; it < SCAN_LOOKBACK_LIMIT; ++it) {
                        vj = *(volatile const uint32_t*)&status[j];
                        if (vj & (SCAN_AGG | SCAN_PRE)) break;
                    }
                    if (it == SCAN_LOOKBACK_LIMIT) { ok = false; set_error(S, 6u); break; }
                    excl += (int32_t)(vj & SCAN_VALUE);
                    if (vj & SCAN_PRE) break;
                    --j;
                }
                if (ok) atomicExch(&status[tile], SCAN_PRE | (uint32_t)(excl + agg));
            }
            excl_sh = excl;
            if (gate == 1 && tile == ntiles - 1) S->live = excl + agg;
        }
        __syncthreads();
        int32_t run = excl_sh;
        for (int u = 0; u < SITEMS; ++u) {
            int32_t before = 0, round = 0;
            for (int q = 0; q < ST / 32; ++q) {
                if (q < w) before += warp_tot[u][q];
                round += warp_tot[u][q];
            }
            const int64_t e = base + u * ST + threadIdx.x;
            if (e < n) prefix[e] = run + before + inc[u] - x[u];
            run += round;
        }
    }
    // The last CTA out resets the tile counter and the status words it used.
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&S->scan_done, 1u) == blk.n - 1;
    }
    __syncthreads();
    if (last) {
        for (int32_t j = threadIdx.x; j < ntiles; j += ST) status[j] = 0u;
        if (threadIdx.x == 0) {
            S->scan_tile = 0u;
            S->scan_done = 0u;
        }
        __threadfence();
    }
}

__global__ void __launch_bounds__(ST) scan_kernel(DevState* S, const int32_t* __restrict__ flag, int32_t* prefix,
                                                 uint32_t* status, int gate) {
    pdl_wait();
    scan_kernel_body(S, flag, prefix, status, gate, grid_blk());
}

// Division of parent i into `slot` with id `did` (divide_kernel body,
// lifecycle.cu:140-204); called only for the cells that divide, from the pass
// that otherwise runs the per-cell CO2 flush.
// (hx, hy, hz: the chamber's half extents less one cell radius.)
__device__ __noinline__ void divide_one(DevState* S, int32_t i, int32_t slot, uint64_t did, double hx, double hy,
                                        double hz) {
    const SoA v = S->cur;
    const double a = AGB_CELL_RADIUS;
    const double half0 = __dmul_rn(0.5, __dsub_rn(v.energy[i], AGB_LIFE_DIVISION_ENERGY_COST));
    const double half = half0 > 0.0 ? half0 : 0.0;
    v.energy[i] = half;
    v.energy[slot] = half;
    v.co2_held[i] = 0.0;
    v.co2_held[slot] = 0.0;
    v.biomass[slot] = AGB_CELL_MASS_DRY;
    const uint64_t hsh = splitmix64(splitmix64(did));      // division_axis, lifecycle.cuh:87-99
    const double u = (double)(hsh >> 33) * (1.0 / 2147483648.0) - 1.0;
    const double phi = (double)(hsh & 0xFFFFFFFFull) * (AGB_TWO_PI / 4294967296.0);
    const double uu = __dmul_rn(u, u);
    const double sr = sqrt(uu < 1.0 ? __dsub_rn(1.0, uu) : 0.0);
    const double ax = __dmul_rn(sr, cos(phi)), ay = __dmul_rn(sr, sin(phi)), az = u;
    // Rounded as written in lifecycle.cu:169-171 (no contraction).
    double x = v.x[i], y = v.y[i], z = v.z[i];
    const double ox = __dmul_rn(a, ax), oy = __dmul_rn(a, ay), oz = __dmul_rn(a, az);
    double xs = __dadd_rn(x, ox), ys = __dadd_rn(y, oy), zs = __dadd_rn(z, oz);
    x = __dsub_rn(x, ox); y = __dsub_rn(y, oy); z = __dsub_rn(z, oz);
    xs = xs < -hx ? -hx : (xs > hx ? hx : xs);
    ys = ys < -hy ? -hy : (ys > hy ? hy : ys);
    zs = zs < -hz ? -hz : (zs > hz ? hz : zs);
    x = x < -hx ? -hx : (x > hx ? hx : x);
    y = y < -hy ? -hy : (y > hy ? hy : y);
    z = z < -hz ? -hz : (z > hz ? hz : z);
    v.x[slot] = xs; v.y[slot] = ys; v.z[slot] = zs;
    v.x[i] = x; v.y[i] = y; v.z[i] = z;
    v.vx[slot] = v.vx[i]; v.vy[slot] = v.vy[i]; v.vz[slot] = v.vz[i];
    v.id[slot] = did;
    v.flags[slot] = v.flags[i];
    v.death_cause[slot] = AGB_DEATH_NONE;
    v.temp_cell[slot] = v.temp_cell[i];
    v.emit_power[slot] = 0.0f;
    v.dir_x[slot] = v.dir_x[i]; v.dir_y[slot] = v.dir_y[i]; v.dir_z[slot] = v.dir_z[i];
    v.age_s[slot] = 0.0f;
    v.rng_state[slot] = pcg_split(v.rng_state[i], did);
    v.taxis_memory[slot] = 0.0f;
    v.run_timer[slot] = 0.0f;
    v.t_local[slot] = v.t_local[i];
    v.irradiance[slot] = 0.0f;
    v.co2_local[slot] = v.co2_local[i];
    v.n2_local[slot] = v.n2_local[i];
}

// ---------------------------------------------------------------------------
// Division (divide_kernel, lifecycle.cu:140-204). Rare per cell, so the
// placement arithmetic stays in FP64 exactly as the reference has it.
// ---------------------------------------------------------------------------
__device__ void life_finalize(DevState* S, int32_t capacity, int32_t compaction_allowed);

//
// With `demand` set (a CO2 grid), the same pass first runs the CO2 flush
// (flush_kernel, lifecycle.cu:235, restricted to the voxels cells sit in: only
// uptake deposited this tick, into exactly those) from each parent's position
// before division moves it, and clears the rationing demand there.
__device__ __forceinline__ void divide_kernel_body(DevState* S, const Ctx& c, const int32_t* __restrict__ divflag,
                                                   const int32_t* __restrict__ prefix, int32_t compaction_allowed,
                                                   unsigned long long* demand, const int32_t* __restrict__ vox,
                                                   Blk blk) {
    const int32_t births_now = S->births;
    const SoA v = S->cur;
    const int32_t n = S->count;                 // base = old count
    const uint64_t first_id = S->next_id;
    const GridDev C2 = c.g[AGB_FIELD_CO2];
    AGB_FOR_CELLS_B(i, blk, (births_now > 0 || demand) ? n : 0) {
        // Only cells that booked demand this tick can have left a deposit or a
        // demand word, so the cells the demand pass marked -1 have nothing to fold.
        const int64_t idx = !demand || !(v.flags[i] & AGB_FLAG_OCCUPIED) ? -1
                            : vox ? (int64_t)vox[i]
                                  : grid_nearest(C2, (float)v.x[i], (float)v.y[i], (float)v.z[i]);
        if (idx >= 0) {
            const unsigned long long raw = atomicExch(&C2.deposit[idx], 0ull);
            if (raw != 0ull) C2.value[idx] = fa(C2.value[idx], fixed_to_f((long long)raw, C2.inv_scale_f, C2.inv_scale_lo, C2.scale));
            demand[idx] = 0ull;
        }
        if (births_now <= 0 || !divflag[i]) continue;
        const int32_t slot = n + prefix[i];
        if (slot >= c.capacity) continue;       // store full: skip, do not wrap
        divide_one(S, i, slot, first_id + (uint64_t)prefix[i], 0.5 * c.chamber_w - AGB_CELL_RADIUS,
                   0.5 * c.chamber_h - AGB_CELL_RADIUS, 0.5 * c.chamber_d - AGB_CELL_RADIUS);
    }
    // The last CTA to finish runs the tick's bookkeeping (every division of
    // this pass has been written by then).
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&S->fin_count, 1u) == blk.n - 1) {
            __threadfence();
            life_finalize(S, c.capacity, compaction_allowed);
            S->fin_count = 0u;
        }
    }
}

__global__ void __launch_bounds__(256) divide_kernel(DevState* S, Ctx c, const int32_t* __restrict__ divflag,
                                                     const int32_t* __restrict__ prefix,
                                                     int32_t compaction_allowed, unsigned long long* demand,
                                                     const int32_t* __restrict__ vox) {
    pdl_wait();
    divide_kernel_body(S, c, divflag, prefix, compaction_allowed, demand, vox, grid_blk());
}

// The host bookkeeping of lifecycle_step (lifecycle.cu:250-293), on the device.
__device__ void life_finalize(DevState* S, int32_t capacity, int32_t compaction_allowed) {
    int32_t births = S->births;
    const int32_t deads = S->deads;
    const int32_t n = S->count;
    const int32_t new_deaths = deads - S->dead_slots_prev;
    if (new_deaths > 0) S->deaths_total += new_deaths;
    if (births > 0) {
        if (n + births > capacity) births = capacity - n;
        if (births > 0) {
            S->divisions_this_window += births;
            S->next_id += (uint64_t)births;
            S->count = n + births;
        }
    }
    const int32_t compact = (compaction_allowed && deads > 0) ? 1 : 0;
    S->compact_now = compact;
    S->dead_slots_prev = compact ? 0 : deads;
    S->births = 0;
    S->deads = 0;
}

// ---------------------------------------------------------------------------
// Compaction (cell_store.cu:368-456): keep = OCCUPIED && ALIVE, stable by
// prefix, gathered out of place into the spare SoA in one fused pass over all
// 25 arrays, then the SoA pointers swap on the device.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void keep_kernel_body(DevState* S, int32_t* keep, Blk blk) {
    if (!S->compact_now) return;
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS_B(i, blk, n) {
        const uint32_t f = v.flags[i];
        keep[i] = ((f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE)) ? 1 : 0;
    }
}

__global__ void __launch_bounds__(256) keep_kernel(DevState* S, int32_t* keep) {
    pdl_wait();
    keep_kernel_body(S, keep, grid_blk());
}

__device__ __forceinline__ void scatter_src_kernel_body(DevState* S, const int32_t* __restrict__ keep,
                                                        const int32_t* __restrict__ prefix, int32_t* src, Blk blk) {
    if (!S->compact_now) return;
    const int32_t n = S->count;
    AGB_FOR_CELLS_B(i, blk, n) {
        if (keep[i]) src[prefix[i]] = i;
    }
}

__global__ void __launch_bounds__(256) scatter_src_kernel(DevState* S, const int32_t* __restrict__ keep,
                                                         const int32_t* __restrict__ prefix, int32_t* src) {
    pdl_wait();
    scatter_src_kernel_body(S, keep, prefix, src, grid_blk());
}

__device__ __forceinline__ void gather_kernel_body(DevState* S, const int32_t* __restrict__ src, Blk blk) {
    if (!S->compact_now) return;
    const int32_t live = S->live;
    if (live >= S->count) return;
    const SoA a = S->cur;
    const SoA b = S->spare;
    AGB_FOR_CELLS_B(k, blk, live) {
        const int32_t i = src[k];
        b.id[k] = a.id[i]; b.flags[k] = a.flags[i]; b.death_cause[k] = a.death_cause[i];
        b.x[k] = a.x[i]; b.y[k] = a.y[i]; b.z[k] = a.z[i];
        b.vx[k] = a.vx[i]; b.vy[k] = a.vy[i]; b.vz[k] = a.vz[i];
        b.energy[k] = a.energy[i]; b.temp_cell[k] = a.temp_cell[i]; b.emit_power[k] = a.emit_power[i];
        b.dir_x[k] = a.dir_x[i]; b.dir_y[k] = a.dir_y[i]; b.dir_z[k] = a.dir_z[i];
        b.biomass[k] = a.biomass[i]; b.co2_held[k] = a.co2_held[i]; b.age_s[k] = a.age_s[i];
        b.rng_state[k] = a.rng_state[i]; b.taxis_memory[k] = a.taxis_memory[i];
        b.run_timer[k] = a.run_timer[i]; b.t_local[k] = a.t_local[i]; b.irradiance[k] = a.irradiance[i];
        b.co2_local[k] = a.co2_local[i]; b.n2_local[k] = a.n2_local[i];
    }
}

__global__ void __launch_bounds__(256) gather_kernel(DevState* S, const int32_t* __restrict__ src) {
    pdl_wait();
    gather_kernel_body(S, src, grid_blk());
}

__device__ __forceinline__ void swap_kernel_body(DevState* S, Blk blk) {
    if (!S->compact_now) return;
    const int32_t live = S->live;
    if (live < S->count) {
        const SoA t = S->cur;
        S->cur = S->spare;
        S->spare = t;
        S->count = live;
    }
    S->compact_now = 0;
}

__global__ void swap_kernel(DevState* S) {
    pdl_wait();
    swap_kernel_body(S, grid_blk());
}

__global__ void force_compact_kernel(DevState* S) {
    pdl_wait(); S->compact_now = 1; }

// ---------------------------------------------------------------------------
// Telemetry (stats_cells_kernel / stats_field_kernel, stats.cu:27-60):
// warp-shuffle sums, one atomic per warp and accumulator. Integer sums, so the
// result is independent of the reduction order, as in the reference.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
    return x;
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long x) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_down_sync(0xFFFFFFFFu, x, o);
        x = y > x ? y : x;
    }
    return x;
}

__global__ void __launch_bounds__(256) stats_cells_kernel(DevState* S, unsigned long long* acc) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->count;
    unsigned long long energy = 0, temp = 0, na = 0, nd = 0, nw = 0, ns = 0;
    AGB_FOR_CELLS(i, n) {
        const uint32_t f = v.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED)) continue;
        const bool alive = (f & AGB_FLAG_ALIVE) != 0u, awake = (f & AGB_FLAG_AWAKE) != 0u;
        na += alive; nd += !alive; nw += awake; ns += !awake;
        energy += (unsigned long long)llround(v.energy[i] * AGB_DEPOSIT_SCALE_STATS);
        if (alive) temp += (unsigned long long)llround((double)v.temp_cell[i] * AGB_DEPOSIT_SCALE_STATS);
    }
    energy = warp_sum(energy); temp = warp_sum(temp);
    na = warp_sum(na); nd = warp_sum(nd); nw = warp_sum(nw); ns = warp_sum(ns);
    if ((threadIdx.x & 31) == 0) {
        if (energy) atomicAdd(&acc[0], energy);
        if (temp) atomicAdd(&acc[1], temp);
        if (na) atomicAdd(&acc[7], na);
        if (nd) atomicAdd(&acc[8], nd);
        if (nw) atomicAdd(&acc[9], nw);
        if (ns) atomicAdd(&acc[10], ns);
    }
}

__global__ void __launch_bounds__(256) stats_field_kernel(const float* __restrict__ val, int64_t count,
                                                          double scale, unsigned long long* sum,
                                                          unsigned long long* mx) {
    pdl_wait();
    unsigned long long s = 0, m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long q = (unsigned long long)llround((double)val[i] * scale);
        s += q;
        if (mx && q > m) m = q;
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(sum, s);
    if (mx) {
        m = warp_max(m);
        if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
    }
}

// ---------------------------------------------------------------------------
// Seeded spawn (spawn_kernel, cell_store.cu:42-130, plus the extension
// placements of include/agb.h). FP64, run once per population.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) spawn_kernel(DevState* S, Ctx c, agb_spawn p) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t base = S->count;
    const uint64_t first_id = S->next_id;
    const double cw = c.chamber_w, ch = c.chamber_h, cd = c.chamber_d, a = AGB_CELL_RADIUS;
    AGB_FOR_CELLS(i, p.count) {
        const int32_t slot = base + i;
        const uint64_t id = first_id + (uint64_t)i;
        Pcg r{cell_rng_init(c.seed, id), cell_stream_inc(id)};
        double x = 0.0, y = 0.0, z = 0.0;
        bool z_done = false;
        switch (p.placement) {
            case AGB_PLACE_GAUSSIAN: {
                double gx, gy;
                gaussian_pair_d(r, gx, gy);
                x = __dadd_rn(p.place_x, __dmul_rn(p.place_radius, gx));
                y = __dadd_rn(p.place_y, __dmul_rn(p.place_radius, gy));
                break;
            }
            case AGB_PLACE_DISC: {
                const double rad = __dmul_rn(p.place_radius, sqrt(uniform01d(r)));
                const double ang = uniform_range(r, 0.0, AGB_TWO_PI);
                x = __dadd_rn(p.place_x, __dmul_rn(rad, cos(ang)));
                y = __dadd_rn(p.place_y, __dmul_rn(rad, sin(ang)));
                break;
            }
            case AGB_PLACE_GRID: {
                const int side = (int)ceil(sqrt((double)p.count));
                const int gx = i % side, gy = i / side;
                x = ((double)gx / side - 0.5) * cw * 0.98;
                y = ((double)gy / side - 0.5) * ch * 0.98;
                break;
            }
            case AGB_PLACE_SLAB_X:
                x = uniform_range(r, p.place_x - p.place_radius, p.place_x + p.place_radius);
                y = uniform_range(r, -0.5 * ch, 0.5 * ch);
                break;
            case AGB_PLACE_CLUSTERS: {
                int32_t k = (int32_t)(uniform01d(r) * (double)p.clusters);
                if (k >= p.clusters) k = p.clusters - 1;
                const uint64_t cid = 0xC1A5C1A5ull + (uint64_t)k;
                Pcg cr{cell_rng_init(c.seed ^ 0x5EEDC1A5ull, cid), cell_stream_inc(cid)};
                const double h = 0.5 * p.cluster_extent;
                const double cx = uniform_range(cr, -h, h);
                const double cy = uniform_range(cr, -h, h);
                const double cz = uniform_range(cr, -h, h);
                double gx, gy, gz, gw;
                gaussian_pair_d(r, gx, gy);
                gaussian_pair_d(r, gz, gw);
                x = __dadd_rn(cx, __dmul_rn(p.place_radius, gx));
                y = __dadd_rn(cy, __dmul_rn(p.place_radius, gy));
                z = __dadd_rn(cz, __dmul_rn(p.place_radius, gz));
                const double zl = -0.5 * cd + a, zh = 0.5 * cd - a;
                z = z < zl ? zl : (z > zh ? zh : z);
                z_done = true;
                break;
            }
            default:
                x = uniform_range(r, -0.5 * cw, 0.5 * cw);
                y = uniform_range(r, -0.5 * ch, 0.5 * ch);
                break;
        }
        {
            const double xl = -0.5 * cw + a, xh = 0.5 * cw - a, yl = -0.5 * ch + a, yh = 0.5 * ch - a;
            x = x < xl ? xl : (x > xh ? xh : x);
            y = y < yl ? yl : (y > yh ? yh : y);
        }
        if (!z_done) z = uniform_range(r, -0.5 * cd + a, 0.5 * cd - a);
        double charge;
        switch (p.charge_dist) {
            case AGB_DIST_UNIFORM: charge = uniform_range(r, p.charge_a, p.charge_b); break;
            case AGB_DIST_NORMAL: { double g0, g1; gaussian_pair_d(r, g0, g1); charge = __dadd_rn(p.charge_a, __dmul_rn(p.charge_b, g0)); break; }
            case AGB_DIST_LOGNORMAL: { double g0, g1; gaussian_pair_d(r, g0, g1); charge = exp(__dadd_rn(log(p.charge_a), __dmul_rn(p.charge_b, g0))); break; }
            default: charge = p.charge_a; break;
        }
        charge = charge < 0.0 ? 0.0 : (charge > 1.0 ? 1.0 : charge);
        if (p.charge_max > 0.0 && charge > p.charge_max) charge = p.charge_max;
        v.id[slot] = id;
        v.flags[slot] = AGB_FLAG_OCCUPIED | AGB_FLAG_ALIVE | (p.awake ? AGB_FLAG_AWAKE : 0u);
        v.death_cause[slot] = AGB_DEATH_NONE;
        v.x[slot] = x; v.y[slot] = y; v.z[slot] = z;
        v.vx[slot] = 0.0; v.vy[slot] = 0.0; v.vz[slot] = 0.0;
        v.energy[slot] = __dmul_rn(charge, AGB_CELL_ENERGY_MAX);
        v.temp_cell[slot] = (float)(p.awake ? AGB_CELL_TEMP_SETPOINT : AGB_AMBIENT_TEMP_DEFAULT);
        v.emit_power[slot] = 0.0f;
        double dx, dy, dz, dd;                                    // gaussian3
        gaussian_pair_d(r, dx, dy);
        gaussian_pair_d(r, dz, dd);
        const double l = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
        double ux = 0.0, uy = 0.0, uz = 1.0;                      // normalize, vec.cuh:34-37
        if (l > 0.0) { const double il = 1.0 / l; ux = __dmul_rn(dx, il); uy = __dmul_rn(dy, il); uz = __dmul_rn(dz, il); }
        v.dir_x[slot] = (float)ux; v.dir_y[slot] = (float)uy; v.dir_z[slot] = (float)uz;
        v.biomass[slot] = AGB_CELL_MASS_DRY;
        v.co2_held[slot] = 0.0;
        v.age_s[slot] = 0.0f;
        v.rng_state[slot] = r.state;
        v.taxis_memory[slot] = 0.0f;
        v.run_timer[slot] = 0.0f;
        v.t_local[slot] = v.temp_cell[slot];
        v.irradiance[slot] = 0.0f;
        v.co2_local[slot] = 0.0f;
        v.n2_local[slot] = 0.0f;
    }
}

__global__ void spawn_finalize_kernel(DevState* S, int32_t count) {
    pdl_wait();
    S->count += count;
    S->next_id += (uint64_t)count;
}

void launch_scan(DevState* S, const LifeBuffers& b, int32_t capacity, int gate, cudaStream_t s) {
    const int32_t ntiles = (capacity + STILE - 1) / STILE;
    launch_k(scan_kernel, ntiles, ST, 0, s, S, b.flags, b.prefix, reinterpret_cast<uint32_t*>(b.tile_sums), gate);
}

void launch_compact_kernels(DevState* S, const LifeBuffers& b, int32_t capacity, int32_t blocks,
                            cudaStream_t s) {
    launch_k(keep_kernel, blocks, 256, 0, s, S, b.flags);
    launch_scan(S, b, capacity, 1, s);
    launch_k(scatter_src_kernel, blocks, 256, 0, s, S, b.flags, b.prefix, b.src);
    launch_k(gather_kernel, blocks, 256, 0, s, S, b.src);
    launch_k(swap_kernel, 1, 1, 0, s, S);
}

AGB_BATCHED_MB(uptake_mark_batch, 256, 4,
            uptake_mark_kernel_body(a.S, a.c, a.p, a.demand, a.gv, a.life.co2_want, a.life.co2_vox, a.life.flags,
                                    blk))
AGB_BATCHED_MB(divide_batch, 256, 4,
            divide_kernel_body(a.S, a.c, a.life.flags, a.life.prefix, a.arg, a.demand, a.life.co2_vox, blk))
AGB_BATCHED(keep_batch, 256, keep_kernel_body(a.S, a.life.flags, blk))
AGB_BATCHED(scatter_src_batch, 256, scatter_src_kernel_body(a.S, a.life.flags, a.life.prefix, a.life.src, blk))
AGB_BATCHED(gather_batch, 256, gather_kernel_body(a.S, a.life.src, blk))
AGB_BATCHED(swap_batch, 32, if (threadIdx.x == 0) swap_kernel_body(a.S, blk))

__global__ void __launch_bounds__(ST) scan_batch(const ChamberArgs* __restrict__ tab,
                                                 const uint32_t* __restrict__ map, int32_t gate) {
    pdl_wait();
    int32_t ch, x;
    batch_block(map, ch, x);
    const ChamberArgs& a = tab[ch];
    scan_kernel_body(a.S, a.life.flags, a.life.prefix, reinterpret_cast<uint32_t*>(a.life.tile_sums), gate,
                     Blk{x, a.nblk});
}

}  // namespace

int32_t scan_blocks(int32_t capacity) { return (capacity + STILE - 1) / STILE; }

bool launch_batched_life(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                         cudaStream_t s) {
    const unsigned g = (unsigned)blocks;
    switch (st) {
        case BStage::UptakeMark: launch_k(uptake_mark_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Scan: launch_k(scan_batch, g, ST, 0, s, tab, map, arg); return true;
        case BStage::Divide: launch_k(divide_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Keep: launch_k(keep_batch, g, 256, 0, s, tab, map); return true;
        case BStage::ScatterSrc: launch_k(scatter_src_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Gather: launch_k(gather_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Swap: launch_k(swap_batch, g, 32, 0, s, tab, map); return true;
        default: return false;
    }
}

void launch_lifecycle(DevState* S, const Ctx& c, const TickParams& p, const LifeBuffers& b,
                      bool compaction_allowed, int32_t blocks, cudaStream_t s, bool demand_done) {
    const GridDev& C2 = c.g[AGB_FIELD_CO2];
    unsigned long long* dem = C2.enabled ? b.co2_demand : nullptr;
    const double gv = C2.enabled ? C2.dx * C2.dx * C2.dz_eff : 0.0;
    if (C2.enabled && !demand_done)
        launch_k(demand_kernel, blocks, 256, 0, s, S, c, p, dem, gv, b.co2_want, b.co2_vox);
    launch_k(uptake_mark_kernel, blocks, 256, 0, s, S, c, p, dem, gv, (const double*)b.co2_want,
             (const int32_t*)b.co2_vox, b.flags);
    launch_scan(S, b, c.capacity, 0, s);
    launch_k(divide_kernel, blocks, 256, 0, s, S, c, b.flags, b.prefix, compaction_allowed ? 1 : 0, dem,
             (const int32_t*)b.co2_vox);
    // Compaction cannot run on this tick unless the host-side period allows it.
    if (compaction_allowed) launch_compact_kernels(S, b, c.capacity, blocks, s);
}

void launch_compact(DevState* S, const Ctx& c, const LifeBuffers& b, int32_t blocks, cudaStream_t s) {
    launch_k(force_compact_kernel, 1, 1, 0, s, S);
    launch_compact_kernels(S, b, c.capacity, blocks, s);
}

void launch_stats(DevState* S, const Ctx& c, unsigned long long* acc, int32_t blocks, cudaStream_t s) {
    cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 12, s);
    launch_k(stats_cells_kernel, blocks, 256, 0, s, S, acc);
    const GridDev& T = c.g[AGB_FIELD_TEMPERATURE];
    const GridDev& C2 = c.g[AGB_FIELD_CO2];
    const GridDev& N2 = c.g[AGB_FIELD_N2];
    auto nb = [](int64_t n) { const int64_t b = (n + 255) / 256; return (unsigned)(b > 2048 ? 2048 : (b < 1 ? 1 : b)); };
    if (T.enabled) launch_k(stats_field_kernel, nb(T.count), 256, 0, s, T.value, T.count, AGB_DEPOSIT_SCALE_STATS, &acc[2], &acc[5]);
    if (C2.enabled) launch_k(stats_field_kernel, nb(C2.count), 256, 0, s, C2.value, C2.count, AGB_STATS_SCALE_FIELD, &acc[3], nullptr);
    if (N2.enabled) launch_k(stats_field_kernel, nb(N2.count), 256, 0, s, N2.value, N2.count, AGB_STATS_SCALE_FIELD, &acc[4], nullptr);
}

void launch_spawn(DevState* S, const Ctx& c, const agb_spawn& p, int32_t blocks, cudaStream_t s) {
    launch_k(spawn_kernel, blocks, 256, 0, s, S, c, p);
    launch_k(spawn_finalize_kernel, 1, 1, 0, s, S, p.count);
}

// Every occupied slot's store set to one energy (set_charge_kernel,
// cell_store.cu:281-297).
__global__ void __launch_bounds__(256) set_charge_kernel(DevState* S, double energy) {
    pdl_wait();
    const SoA v = S->cur;
    AGB_FOR_CELLS(i, S->count) {
        if (v.flags[i] & AGB_FLAG_OCCUPIED) v.energy[i] = energy;
    }
}

void launch_set_charge(DevState* S, double energy, int32_t blocks, cudaStream_t s) {
    launch_k(set_charge_kernel, blocks, 256, 0, s, S, energy);
}

}  // namespace agb
