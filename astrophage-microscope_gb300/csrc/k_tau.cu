// k_tau.cu -- Taumoeba, the predator (src/sim/predation.cu): spawn, hunt,
// claim resolution, nitrogen lethality, division and compaction.
//
// The predator population is small (at most 65,536), so its arithmetic is the
// reference's FP64 arithmetic, operation by operation (explicitly rounded, no
// contraction). The per-world constants that the reference recomputes in
// every thread (the OU step of a fixed mass under a fixed drag at the ambient
// temperature, the run-and-tumble memory weight) come from the host in FP64
// (TauParams). Division and compaction run in one CTA that walks the store in
// chunks of 1024 predators with a block scan, so daughter slots and ids follow
// the reference's exclusive prefix sums and nothing synchronises with the host.
#include <cuda_runtime.h>

#include "cells.h"
#include "kernels.h"

namespace agb {

namespace {

constexpr int TAU_BLOCK = 256;
constexpr int LIFE_THREADS = 1024;

__device__ __forceinline__ double dot3d(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// normalize (vec.cuh:34-37): a * (1 / |a|), or +z for the zero vector.
__device__ __forceinline__ void normalize3d(double& x, double& y, double& z) {
    const double l = sqrt(dot3d(x, y, z));
    if (l > 0.0) {
        const double inv = __drcp_rn(l);
        x = __dmul_rn(x, inv); y = __dmul_rn(y, inv); z = __dmul_rn(z, inv);
    } else {
        x = 0.0; y = 0.0; z = 1.0;
    }
}

// gaussian3 (rng.cuh:111-117): two pairs, the fourth variate unused.
__device__ __forceinline__ void gaussian3d(Pcg& r, double& x, double& y, double& z) {
    double d;
    gaussian_pair_d(r, x, y);
    gaussian_pair_d(r, z, d);
}

// ou_advance_axis (integrator.cuh:128-154) with the per-world coefficients.
__device__ __forceinline__ void ou_axis_d(double& pos, double& vel, double force, const TauParams& p, double z1,
                                          double z2) {
    const double v_term = __ddiv_rn(force, p.gamma);
    const double dpos = __dadd_rn(__dmul_rn(v_term, p.dt), __dmul_rn(__dmul_rn(__dsub_rn(vel, v_term), p.ome), p.inv_beta));
    const double dvel = __dmul_rn(__dsub_rn(v_term, vel), p.ome);
    double npos = __dadd_rn(pos, dpos);
    double nvel = __dadd_rn(vel, dvel);
    if (p.noise && p.s_rr > 0.0) {
        npos = __dadd_rn(npos, __dmul_rn(p.s_rr, z1));
        nvel = __dadd_rn(nvel, __dadd_rn(__dmul_rn(p.noise_a, z1), __dmul_rn(p.noise_b, z2)));
    } else if (p.noise) {
        nvel = __dadd_rn(nvel, __dmul_rn(p.s_vv, z2));
    }
    pos = npos;
    vel = nvel;
}

// apply_boundary_axis (integrator.cuh:233-254); the predator ignores "culled".
__device__ __forceinline__ void tau_wall(double& pos, double& vel, const TauParams& p, int ax, int mode) {
    if (pos >= p.lo[ax] && pos <= p.hi[ax]) return;
    if (mode == AGB_WALL_PERIODIC) {
        for (int k = 0; k < 64 && pos < -p.half[ax]; ++k) pos = __dadd_rn(pos, p.span[ax]);
        for (int k = 0; k < 64 && pos > p.half[ax]; ++k) pos = __dsub_rn(pos, p.span[ax]);
        return;
    }
    if (mode == AGB_WALL_ABSORBING) return;
    pos = pos < p.lo[ax] ? p.lo[ax] : p.hi[ax];
    vel = 0.0;
}

// spawn_kernel (predation.cu:33-74).
__global__ void __launch_bounds__(TAU_BLOCK) tau_spawn_kernel(TauState* T, int32_t count, uint64_t seed, TauParams p) {
    pdl_wait();
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const TauSoA v = T->cur;
    const int32_t slot = T->count + i;
    if (slot >= T->capacity) return;
    const uint64_t id = T->next_id + (uint64_t)i;
    Pcg r{cell_rng_init(splitmix64(seed), id), cell_stream_inc(id)};
    v.x[slot] = uniform_range(r, p.lo[0], p.hi[0]);
    v.y[slot] = uniform_range(r, p.lo[1], p.hi[1]);
    v.z[slot] = uniform_range(r, p.lo[2], p.hi[2]);
    v.vx[slot] = 0.0; v.vy[slot] = 0.0; v.vz[slot] = 0.0;
    double dx, dy, dz;
    gaussian3d(r, dx, dy, dz);
    normalize3d(dx, dy, dz);
    v.dir_x[slot] = (float)dx; v.dir_y[slot] = (float)dy; v.dir_z[slot] = (float)dz;
    v.id[slot] = id;
    v.flags[slot] = AGB_FLAG_OCCUPIED | AGB_FLAG_ALIVE;
    v.biomass[slot] = AGB_TAU_MASS_DRY;
    v.prey_biomass[slot] = 0.0;
    v.digest_timer[slot] = 0.0f;
    v.tolerance[slot] = (float)AGB_TAU_N2_TOLERANCE_INIT;
    v.generation[slot] = 0u;
    v.rng_state[slot] = r.state;
    v.density_ema[slot] = 0.0f;
    v.run_timer[slot] = 0.0f;
    v.target[slot] = -1;
}

__global__ void tau_spawn_finalize_kernel(TauState* T, int32_t count) {
    pdl_wait();
    const int32_t room = T->capacity - T->count;
    const int32_t n = count < room ? count : room;
    T->count += n;
    T->next_id += (uint64_t)n;
}

// The per-cell claim word: all ones, so atomicMin resolves to the lowest id.
__global__ void __launch_bounds__(TAU_BLOCK) tau_claim_reset_kernel(unsigned long long* claim, int32_t n) {
    pdl_wait();
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        claim[i] = ~0ull;
}

// hunt_kernel (predation.cu:80-158): sense the live prey around the predator
// and the first overlapping one in hash order (the walk of
// ASTRO_FOR_EACH_NEIGHBOUR, hash.cuh:88-111, over this tick's cell hash, with
// the cells' current positions), claim it when hunting, run and tumble on the
// prey count, crawl one OU step, walls, digestion on the biology clock.
__global__ void __launch_bounds__(TAU_BLOCK) tau_hunt_kernel(TauState* T, DevState* S, HashDev h, TauParams p,
                                                             unsigned long long* claim) {
    pdl_wait();
    const TauSoA t = T->cur;
    const int32_t n = T->count;
    const SoA c = S->cur;
    const double rr = __dmul_rn(AGB_TAU_RADIUS + AGB_CELL_RADIUS, AGB_TAU_RADIUS + AGB_CELL_RADIUS);
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t f = t.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        double px = t.x[i], py = t.y[i], pz = t.z[i];
        const bool digesting = t.digest_timer[i] > 0.0f;
        int32_t prey_count = 0, prey = -1;
        int32_t gx, gy, gz;
        hash_coords(h, px, py, pz, gx, gy, gz);
        for (int32_t dz = -1; dz <= 1; ++dz) {
            const int32_t cz = gz + dz;
            if (cz < 0 || cz >= h.nz) continue;
            for (int32_t dy = -1; dy <= 1; ++dy) {
                const int32_t cy = gy + dy;
                if (cy < 0 || cy >= h.ny) continue;
                for (int32_t dx = -1; dx <= 1; ++dx) {
                    const int32_t cx = gx + dx;
                    if (cx < 0 || cx >= h.nx) continue;
                    const int2 rg = h.ranges[(cz * h.ny + cy) * h.nx + cx];
                    for (int32_t k = rg.x; k < rg.y; ++k) {
                        const int32_t j = (int32_t)h.vals_sorted[k];
                        const uint32_t cf = c.flags[j];
                        if (!(cf & AGB_FLAG_OCCUPIED) || !(cf & AGB_FLAG_ALIVE)) continue;
                        ++prey_count;
                        if (prey < 0 && dot3d(__dsub_rn(px, c.x[j]), __dsub_rn(py, c.y[j]), __dsub_rn(pz, c.z[j])) < rr)
                            prey = j;
                    }
                }
            }
        }
        if (!digesting && prey >= 0) {
            t.target[i] = prey;
            atomicMin(&claim[prey], (unsigned long long)t.id[i]);
        } else {
            t.target[i] = -1;
        }
        // tau_should_tumble (predation.cuh:36-41)
        Pcg rng{t.rng_state[i], cell_stream_inc(t.id[i])};
        float ema = t.density_ema[i];
        float run = t.run_timer[i];
        double ux = (double)t.dir_x[i], uy = (double)t.dir_y[i], uz = (double)t.dir_z[i];
        const double delta = __dsub_rn((double)(float)prey_count, (double)ema);
        ema = (float)__dadd_rn((double)ema, __dmul_rn(p.alpha, delta));
        if (!(delta > 0.0 && (double)run < AGB_TAXIS_RUN_MAX)) {
            gaussian3d(rng, ux, uy, uz);
            normalize3d(ux, uy, uz);
            run = 0.0f;
        } else {
            run = __fadd_rn(run, p.dt_f);
        }
        t.density_ema[i] = ema;
        t.run_timer[i] = run;
        t.dir_x[i] = (float)ux; t.dir_y[i] = (float)uy; t.dir_z[i] = (float)uz;
        // integrate_cell (integrator.cuh:159-169) with the crawl thrust along the heading
        double vx = t.vx[i], vy = t.vy[i], vz = t.vz[i];
        double z1, z2, z3, z4, z5, z6;
        gaussian_pair_d(rng, z1, z2);
        gaussian_pair_d(rng, z3, z4);
        gaussian_pair_d(rng, z5, z6);
        ou_axis_d(px, vx, __dmul_rn(ux, AGB_TAU_CRAWL_THRUST), p, z1, z2);
        ou_axis_d(py, vy, __dmul_rn(uy, AGB_TAU_CRAWL_THRUST), p, z3, z4);
        ou_axis_d(pz, vz, __dmul_rn(uz, AGB_TAU_CRAWL_THRUST), p, z5, z6);
        t.rng_state[i] = rng.state;
        tau_wall(px, vx, p, 0, p.boundary_x);
        tau_wall(py, vy, p, 1, p.boundary_y);
        tau_wall(pz, vz, p, 2, AGB_WALL_REFLECTING);
        t.x[i] = px; t.y[i] = py; t.z[i] = pz;
        t.vx[i] = vx; t.vy[i] = vy; t.vz[i] = vz;
        if (digesting) {
            float d = __fsub_rn(t.digest_timer[i], p.dt_bio_f);
            if (d <= 0.0f) {
                t.biomass[i] = __dadd_rn(t.biomass[i], __dmul_rn(t.prey_biomass[i], AGB_TAU_BIOMASS_YIELD));
                t.prey_biomass[i] = 0.0;
                d = 0.0f;
            }
            t.digest_timer[i] = d;
        }
    }
}

// resolve_kernel (predation.cu:160-182): the winning predator engulfs its prey.
__global__ void __launch_bounds__(TAU_BLOCK) tau_resolve_kernel(TauState* T, DevState* S, TauParams p,
                                                                const unsigned long long* __restrict__ claim) {
    pdl_wait();
    const TauSoA t = T->cur;
    const int32_t n = T->count;
    const SoA c = S->cur;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t prey = t.target[i];
        if (prey < 0 || claim[prey] != (unsigned long long)t.id[i]) continue;
        const uint32_t cf = c.flags[prey];
        if (!(cf & AGB_FLAG_OCCUPIED) || !(cf & AGB_FLAG_ALIVE)) continue;
        c.flags[prey] = cf & ~AGB_FLAG_ALIVE;
        c.death_cause[prey] = AGB_DEATH_PREDATED;
        c.emit_power[prey] = 0.0f;
        if (p.disposition != AGB_STORE_RETAIN) c.energy[prey] = 0.0;   // corpse_energy
        t.digest_timer[i] = (float)AGB_TAU_DIGEST_TIME;
        t.prey_biomass[i] = c.biomass[prey];
    }
}

// nitrogen_kernel (predation.cu:189-205): one uniform per live predator,
// always drawn; above its tolerance-raised threshold the Poisson hazard kills.
__global__ void __launch_bounds__(TAU_BLOCK) tau_nitrogen_kernel(TauState* T, GridDev n2, TauParams p) {
    pdl_wait();
    const TauSoA t = T->cur;
    const int32_t n = T->count;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t f = t.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        Pcg rng{t.rng_state[i], cell_stream_inc(t.id[i])};
        const double u = uniform01d(rng);
        t.rng_state[i] = rng.state;
        const double n2_local = n2.enabled ? (double)grid_sample(n2, n2.value, (float)t.x[i], (float)t.y[i],
                                                                  (float)t.z[i]) : 0.0;
        const double thr = __dmul_rn(AGB_TAU_N2_LETHAL_CONC,
                                     __dadd_rn(1.0, __dmul_rn((double)t.tolerance[i], AGB_TAU_N2_TOLERANCE_K)));
        const double hz = __dsub_rn(n2_local, thr);
        const double hazard = hz > 0.0 ? hz : 0.0;
        const double prob = -expm1(__dmul_rn(__dmul_rn(-hazard, AGB_TAU_N2_HAZARD_RATE), p.dt_bio));
        if (u < prob) t.flags[i] = f & ~AGB_FLAG_ALIVE;
    }
}

// Exclusive scan of one 0/1 flag per thread over the CTA; returns the
// thread's prefix and, through `total`, the CTA's sum.
__device__ __forceinline__ int32_t cta_exclusive_scan(int32_t flag, int32_t* warp_tot, int32_t& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, flag != 0);
    const int32_t in_warp = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) warp_tot[wid] = __popc(bal);
    __syncthreads();
    int32_t before = 0, sum = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        const int32_t v = warp_tot[k];
        if (k < wid) before += v;
        sum += v;
    }
    __syncthreads();
    total = sum;
    return before + in_warp;
}

__device__ __forceinline__ double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// The store's 20 arrays of slot `from` copied to slot `to` of `dst`.
__device__ __forceinline__ void tau_copy(const TauSoA& s, int32_t from, const TauSoA& d, int32_t to) {
    d.id[to] = s.id[from]; d.flags[to] = s.flags[from];
    d.x[to] = s.x[from]; d.y[to] = s.y[from]; d.z[to] = s.z[from];
    d.vx[to] = s.vx[from]; d.vy[to] = s.vy[from]; d.vz[to] = s.vz[from];
    d.dir_x[to] = s.dir_x[from]; d.dir_y[to] = s.dir_y[from]; d.dir_z[to] = s.dir_z[from];
    d.biomass[to] = s.biomass[from]; d.prey_biomass[to] = s.prey_biomass[from];
    d.digest_timer[to] = s.digest_timer[from]; d.tolerance[to] = s.tolerance[from];
    d.generation[to] = s.generation[from]; d.rng_state[to] = s.rng_state[from];
    d.density_ema[to] = s.density_ema[from]; d.run_timer[to] = s.run_timer[from];
    d.target[to] = s.target[from];
}

// Division (tau_mark_kernel + tau_divide_kernel, predation.cu:211-284) and
// compaction (taumoeba_store_compact, predation.cu:486-521) in one CTA.
// Division: the predators whose dry biomass reached the threshold split in
// prefix order into slots count + prefix (those past capacity are skipped),
// the daughter's tolerance mutated by the first draw of its own stream.
// Compaction (when enabled and a predator was dead before the divisions):
// the live predators are packed in order into the spare arrays, which become
// the store.
__global__ void __launch_bounds__(LIFE_THREADS) tau_life_kernel(TauState* T, TauParams p) {
    pdl_wait();
    __shared__ int32_t warp_tot[LIFE_THREADS / 32];
    __shared__ int32_t s_deads;
    const TauSoA t = T->cur;
    const int32_t n = T->count, cap = T->capacity;
    const uint64_t first_id = T->next_id;
    if (threadIdx.x == 0) s_deads = 0;
    __syncthreads();
    int32_t carry = 0, deads = 0;
    for (int32_t c0 = 0; c0 < n; c0 += blockDim.x) {
        const int32_t i = c0 + threadIdx.x;
        bool divides = false;
        if (i < n) {
            const uint32_t f = t.flags[i];
            const bool occ = (f & AGB_FLAG_OCCUPIED) != 0u, alive = (f & AGB_FLAG_ALIVE) != 0u;
            divides = occ && alive && t.biomass[i] >= AGB_TAU_DIVIDE_BIOMASS;
            deads += (occ && !alive) ? 1 : 0;
        }
        int32_t chunk = 0;
        const int32_t pre = carry + cta_exclusive_scan(divides ? 1 : 0, warp_tot, chunk);
        if (divides && n + pre < cap) {
            const int32_t slot = n + pre;
            const uint64_t did = first_id + (uint64_t)pre;
            const double half = __dmul_rn(0.5, t.biomass[i]);
            t.biomass[i] = half;
            t.biomass[slot] = half;
            Pcg dr{pcg_split(t.rng_state[i], did), cell_stream_inc(did)};
            double mutation, unused;
            gaussian_pair_d(dr, mutation, unused);
            t.tolerance[slot] = (float)clampd(__dadd_rn((double)t.tolerance[i], __dmul_rn(AGB_TAU_MUTATION_SIGMA, mutation)),
                                              0.0, 1.0);
            t.rng_state[slot] = dr.state;
            t.generation[slot] = t.generation[i] + 1u;
            // division_axis (lifecycle.cuh:87-99)
            const uint64_t hsh = splitmix64(splitmix64(did));
            const double u = (double)(hsh >> 33) * (1.0 / 2147483648.0) - 1.0;
            const double phi = (double)(hsh & 0xFFFFFFFFull) * (AGB_TWO_PI / 4294967296.0);
            const double uu = __dmul_rn(u, u);
            const double sr = sqrt(uu < 1.0 ? __dsub_rn(1.0, uu) : 0.0);
            const double ox = __dmul_rn(AGB_TAU_RADIUS, __dmul_rn(sr, cos(phi)));
            const double oy = __dmul_rn(AGB_TAU_RADIUS, __dmul_rn(sr, sin(phi)));
            const double oz = __dmul_rn(AGB_TAU_RADIUS, u);
            const double x = t.x[i], y = t.y[i], z = t.z[i];
            t.x[slot] = clampd(__dadd_rn(x, ox), p.lo[0], p.hi[0]);
            t.y[slot] = clampd(__dadd_rn(y, oy), p.lo[1], p.hi[1]);
            t.z[slot] = clampd(__dadd_rn(z, oz), p.lo[2], p.hi[2]);
            t.x[i] = clampd(__dsub_rn(x, ox), p.lo[0], p.hi[0]);
            t.y[i] = clampd(__dsub_rn(y, oy), p.lo[1], p.hi[1]);
            t.z[i] = clampd(__dsub_rn(z, oz), p.lo[2], p.hi[2]);
            t.id[slot] = did;
            t.flags[slot] = t.flags[i];
            t.vx[slot] = t.vx[i]; t.vy[slot] = t.vy[i]; t.vz[slot] = t.vz[i];
            t.dir_x[slot] = t.dir_x[i]; t.dir_y[slot] = t.dir_y[i]; t.dir_z[slot] = t.dir_z[i];
            t.prey_biomass[slot] = 0.0;
            t.digest_timer[slot] = 0.0f;
            t.density_ema[slot] = 0.0f;
            t.run_timer[slot] = 0.0f;
            t.target[slot] = -1;
        }
        carry += chunk;
    }
    if (deads) atomicAdd(&s_deads, deads);
    __syncthreads();
    const int32_t births = n + carry > cap ? cap - n : carry;
    const int32_t count = n + births;
    if (!(p.compaction && s_deads > 0)) {
        if (threadIdx.x == 0) {
            T->count = count;
            T->next_id = first_id + (uint64_t)births;
        }
        return;
    }
    const TauSoA d = T->spare;
    int32_t live = 0;
    for (int32_t c0 = 0; c0 < count; c0 += blockDim.x) {
        const int32_t i = c0 + threadIdx.x;
        bool keep = false;
        if (i < count) {
            const uint32_t f = t.flags[i];
            keep = (f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE);
        }
        int32_t chunk = 0;
        const int32_t pre = live + cta_exclusive_scan(keep ? 1 : 0, warp_tot, chunk);
        if (keep) tau_copy(t, i, d, pre);
        live += chunk;
    }
    if (threadIdx.x == 0) {
        T->spare = t;
        T->cur = d;
        T->count = live;
        T->next_id = first_id + (uint64_t)births;
    }
}

// stats_taumoeba_kernel (stats.cu:65-73).
__global__ void __launch_bounds__(TAU_BLOCK) tau_stats_kernel(TauState* T, unsigned long long* acc) {
    pdl_wait();
    const TauSoA t = T->cur;
    const int32_t n = T->count;
    unsigned long long cnt = 0, tol = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t f = t.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        ++cnt;
        tol += (unsigned long long)llround(__dmul_rn((double)t.tolerance[i], AGB_DEPOSIT_SCALE_STATS));
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
        tol += __shfl_down_sync(0xFFFFFFFFu, tol, o);
    }
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicAdd(&acc[11], cnt);
        atomicAdd(&acc[6], tol);
    }
}

unsigned tau_blocks(int32_t n) {
    const int32_t b = (n + TAU_BLOCK - 1) / TAU_BLOCK;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

size_t tau_blob_bytes(int32_t cap) {
    auto a = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t c = (size_t)cap;
    return a(8 * c) + a(4 * c) + 6 * a(8 * c) + 3 * a(4 * c) + 2 * a(8 * c) + 2 * a(4 * c) + a(4 * c) + a(8 * c) +
           2 * a(4 * c) + a(4 * c);
}

TauSoA tau_carve(void* blob, int32_t cap) {
    char* q = static_cast<char*>(blob);
    auto take = [&](size_t w) { char* p = q; q += ((size_t)cap * w + 255) / 256 * 256; return (void*)p; };
    TauSoA t;
    t.id = (uint64_t*)take(8); t.flags = (uint32_t*)take(4);
    t.x = (double*)take(8); t.y = (double*)take(8); t.z = (double*)take(8);
    t.vx = (double*)take(8); t.vy = (double*)take(8); t.vz = (double*)take(8);
    t.dir_x = (float*)take(4); t.dir_y = (float*)take(4); t.dir_z = (float*)take(4);
    t.biomass = (double*)take(8); t.prey_biomass = (double*)take(8);
    t.digest_timer = (float*)take(4); t.tolerance = (float*)take(4);
    t.generation = (uint32_t*)take(4); t.rng_state = (uint64_t*)take(8);
    t.density_ema = (float*)take(4); t.run_timer = (float*)take(4);
    t.target = (int32_t*)take(4);
    return t;
}

void launch_tau_spawn(TauState* T, int32_t count, uint64_t seed, const TauParams& p, cudaStream_t s) {
    if (count <= 0) return;
    launch_k(tau_spawn_kernel, tau_blocks(count), TAU_BLOCK, 0, s, T, count, seed, p);
    launch_k(tau_spawn_finalize_kernel, 1, 1, 0, s, T, count);
}

void launch_predation(TauState* T, DevState* S, const HashDev& h, const GridDev& n2, const TauParams& p,
                      unsigned long long* claim, int32_t cell_capacity, int32_t tau_capacity, cudaStream_t s) {
    const unsigned cb = tau_blocks(cell_capacity) < 1024u ? tau_blocks(cell_capacity) : 1024u;
    launch_k(tau_claim_reset_kernel, cb, TAU_BLOCK, 0, s, claim, cell_capacity);
    const unsigned tb = tau_blocks(tau_capacity);
    launch_k(tau_hunt_kernel, tb, TAU_BLOCK, 0, s, T, S, h, p, claim);
    launch_k(tau_resolve_kernel, tb, TAU_BLOCK, 0, s, T, S, p, (const unsigned long long*)claim);
    launch_k(tau_nitrogen_kernel, tb, TAU_BLOCK, 0, s, T, n2, p);
    launch_k(tau_life_kernel, 1, LIFE_THREADS, 0, s, T, p);
}

void launch_tau_stats(TauState* T, int32_t tau_capacity, unsigned long long* acc, cudaStream_t s) {
    launch_k(tau_stats_kernel, tau_blocks(tau_capacity), TAU_BLOCK, 0, s, T, acc);
}

}  // namespace agb
