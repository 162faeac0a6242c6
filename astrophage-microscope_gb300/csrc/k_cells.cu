// k_cells.cu -- per-cell stages of the tick: thermal coupling
// (src/sim/thermal.cu:19-103), occlusion stamp + transmittance sweep + feeding
// (src/sim/emission.cu:17-177) and motion: field sample + forces + exact OU
// integration (src/sim/integrator.cu:20-177).
//
// Forces and integration are two kernels, as in the reference (ADR-018): the
// neighbour walks run in hash-sorted order (warp lanes share bucket
// neighbourhoods), integration in slot order (coalesced state access). The
// walks read the hash's sorted snapshot of positions, so they never see a
// position this tick has already moved.
#include <cuda_runtime.h>

#include "cells.h"

namespace agb {

namespace {

// ASTRO_FOR_EACH_NEIGHBOUR (src/sim/hash.cuh:88-111): buckets in z, y, x
// order, entries in sorted order. The three x-adjacent buckets of a row are
// consecutive keys, hence one contiguous run of the sorted arrays.
//
// skip_axis / skip_side (optional) drop the neighbour buckets one step along
// that axis on that side: the feeding walk uses it for the downstream layer
// under axis-aligned light, whose cells can only lie in the cell's shadow-free
// half-space (see feed_kernel).
//
// lane / L split one walk over L threads: lane j visits entries j, j+L, ...
// of every row (L = 1: the whole walk in one thread).
template <int L = 1, class F>
__device__ __forceinline__ void walk_neighbours(const HashDev& h, int32_t gx, int32_t gy, int32_t gz, F&& f,
                                                int skip_axis = -1, int skip_side = 0, int lane = 0) {
    int32_t xlo = gx > 0 ? gx - 1 : 0;
    int32_t xhi = gx < h.nx - 1 ? gx + 1 : h.nx - 1;
    if (skip_axis == 0) {
        if (skip_side > 0) xhi = gx;
        else xlo = gx;
    }
    const int32_t nxr = xhi - xlo;
    // All nine rows' bucket ranges are loaded before any entry is visited, so
    // the 27 table reads overlap instead of serialising row by row.
    int32_t lo[9], hi[9];
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int32_t oz = r / 3 - 1, oy = r % 3 - 1;
        const int32_t cz = gz + oz, cy = gy + oy;
        lo[r] = 0;
        hi[r] = 0;
        if (cz < 0 || cz >= h.nz || cy < 0 || cy >= h.ny) continue;
        if ((skip_axis == 2 && oz == skip_side) || (skip_axis == 1 && oy == skip_side)) continue;
        const int32_t b0 = (cz * h.ny + cy) * h.nx + xlo;
        // The occupancy bits of the row's 1-3 buckets (one 64-bit window over
        // the bitmap, which stays cache-resident) decide which ranges to load.
        const uint32_t wi = (uint32_t)b0 >> 5, sh = (uint32_t)b0 & 31u;
        const uint64_t win = ((uint64_t)__ldg(&h.occ[wi + 1]) << 32) | __ldg(&h.occ[wi]);
        const uint32_t bits = (uint32_t)(win >> sh) & ((2u << nxr) - 1u);
        if (bits == 0u) continue;
        const int2 r0 = (bits & 1u) ? __ldg(&h.ranges[b0]) : make_int2(0, 0);
        const int2 r1 = (bits & 2u) ? __ldg(&h.ranges[b0 + 1]) : make_int2(0, 0);
        const int2 r2 = (bits & 4u) ? __ldg(&h.ranges[b0 + 2]) : make_int2(0, 0);
        int32_t l = 0, e = 0;
        bool found = false;
        if (r0.y > r0.x) { l = r0.x; e = r0.y; found = true; }
        if (r1.y > r1.x) { if (!found) { l = r1.x; found = true; } e = r1.y; }
        if (r2.y > r2.x) { if (!found) { l = r2.x; found = true; } e = r2.y; }
        lo[r] = l;
        hi[r] = e;
    }
    // Visit entries in order, the next record's load in flight while the
    // current one is evaluated. A row's y and z bucket offsets are fixed, so
    // their part of the separation, (g - b) * cell with g - b in {-1, 0, 1},
    // is passed along as an exact constant (cy, cz).
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const int32_t k0 = lo[r] + lane;
        if (k0 >= hi[r]) continue;
        const float cy = (float)(1 - r % 3) * h.cell_f, cz = (float)(1 - r / 3) * h.cell_f;
        float4 nxt = __ldg(&h.rec[k0]);
        for (int32_t k = k0; k < hi[r]; k += L) {
            const float4 cur = nxt;
            if (k + L < hi[r]) nxt = __ldg(&h.rec[k + L]);
            f(k, cur, cy, cz);
        }
    }
}

// Lanes of one walk group (L consecutive lanes of a warp, L a power of two
// up to 8) and reductions over them. Butterfly order is symmetric, so every
// lane of the group ends with the same bits.
template <int L>
__device__ __forceinline__ unsigned group_mask() {
    if (L == 1) return 1u << (threadIdx.x & 31u);
    return ((1u << L) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(L - 1));
}
template <int L>
__device__ __forceinline__ float group_sum(float v, unsigned m) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o, L);
    return v;
}
template <int L>
__device__ __forceinline__ float group_prod(float v, unsigned m) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v *= __shfl_xor_sync(m, v, o, L);
    return v;
}
template <int L>
__device__ __forceinline__ int32_t group_isum(int32_t v, unsigned m) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o, L);
    return v;
}

__device__ __forceinline__ void unpack_bucket(float w, int32_t& gx, int32_t& gy, int32_t& gz) {
    const uint32_t u = __float_as_uint(w);
    gx = (int32_t)(u & 0x7FFu);
    gy = (int32_t)((u >> 11) & 0x7FFu);
    gz = (int32_t)(u >> 22);
}

// Separation self - other from two snapshot records (FP32, ~2e-7 relative):
// (bucket delta) * cell + (offset delta), one rounding per axis. The walk
// supplies the y and z bucket terms of the row (cy, cz; exact, as the delta
// is -1, 0 or 1), so only the x bucket is unpacked here; the result is the
// same single rounding of the same exact sum.
__device__ __forceinline__ void rec_delta(const HashDev& h, const float4& a, int32_t ax, const float4& b,
                                          float cy, float cz, float& dx, float& dy, float& dz) {
    const int32_t bx = (int32_t)(__float_as_uint(b.w) & 0x7FFu);
    dx = (float)(ax - bx) * h.cell_f + (a.x - b.x);
    dy = cy + (a.y - b.y);
    dz = cz + (a.z - b.z);
}

// ---------------------------------------------------------------------------
// Thermal substep (thermal_kernel, src/sim/thermal.cu:19-71)
// ---------------------------------------------------------------------------
// `first`: the tick's first substep, which finds each cell's voxel from its
// position and keeps it in c.t_vox; the later substeps read it back.
__device__ __forceinline__ void thermal_kernel_body(DevState* S, const Ctx& c, const TickParams& p, bool first,
                                                    Blk blk) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    const GridDev T = c.g[AGB_FIELD_TEMPERATURE];
    bool deposited = false;
    AGB_FOR_CELLS_B(i, blk, n) {
        const uint32_t flags = v.flags[i];
        if (!(flags & AGB_FLAG_OCCUPIED)) continue;
        int64_t idx;
        if (first || !c.t_vox) {
            idx = grid_nearest(T, d2f(v.x[i]), d2f(v.y[i]), d2f(v.z[i]));
            if (c.t_vox) c.t_vox[i] = (int32_t)idx;
        } else {
            idx = c.t_vox[i];
        }
        const float t_grid = T.value[idx];
        bool awake = (flags & AGB_FLAG_AWAKE) != 0u;
        uint32_t nf = flags;
        if (!awake && t_grid >= c.setpoint_up) {          // should_ignite, thermal.cuh:51-53
            awake = true;
            nf = flags | AGB_FLAG_AWAKE;
            v.flags[i] = nf;
        }
        v.temp_cell[i] = awake ? c.setpoint_hi : t_grid;   // (float)cell_temperature
        if (!awake || !(flags & AGB_FLAG_ALIVE)) continue;
        // lumped_exchange_energy (thermal.cuh:80-86): C (T_cell - T_grid) relax,
        // with T_cell - T_grid formed exactly from the setpoint's float pair.
        const float dT = (c.setpoint_hi - t_grid) + c.setpoint_lo;
        const float e = p.t_cap_relax * dT;
        const double E = v.energy[i];
        double En = E - f2d(e);
        float amount = p.t_relax * dT;                    // moved / C when unclamped
        if (dkey(En) < dkey(0.0)) {
            amount = (float)(E / p.t_cap);
            En = 0.0;
        } else if (dkey(En) > dkey(AGB_CELL_ENERGY_MAX)) {
            amount = (float)((E - AGB_CELL_ENERGY_MAX) / p.t_cap);
            En = AGB_CELL_ENERGY_MAX;
        }
        v.energy[i] = En;
        deposit_fixed(&T.deposit[idx], to_fixed_f(amount, T.scale_f));
        deposited = true;
        if (dkey(En) <= dkey(0.0)) {                     // starved
            v.flags[i] = nf & ~AGB_FLAG_ALIVE;
            v.death_cause[i] = AGB_DEATH_STARVED;
            v.emit_power[i] = 0.0f;
        }
    }
    // Only awake, living cells exchange heat; when none did, the flush that
    // follows has nothing to fold in (flush_by_cells_kernel_body skips it).
    if (__syncthreads_or(deposited) && threadIdx.x == 0) S->t_deposited = 1u;
}

__global__ void __launch_bounds__(256) thermal_kernel(DevState* S, Ctx c, TickParams p, int first) {
    pdl_wait();
    thermal_kernel_body(S, c, p, first != 0, grid_blk());
}

// ---------------------------------------------------------------------------
// Emission (src/sim/emission.cu:17-177)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void clear_stamps_kernel_body(DevState* S, const Ctx& c,
                                                         const int32_t* __restrict__ stamp_idx, Blk blk) {
    const int32_t n = S->n_stamps;
    unsigned long long* dep = c.g[AGB_FIELD_IRRADIANCE].deposit;
    uint32_t* bits = c.irr_stamp_bits;
    AGB_FOR_CELLS_B(i, blk, n) {
        const int32_t idx = stamp_idx[i];
        if (idx >= 0) {
            dep[idx] = 0ull;
            if (bits) atomicAnd(&bits[idx >> 5], ~(1u << (idx & 31)));
        }
    }
}

__global__ void clear_stamps_kernel(DevState* S, Ctx c, const int32_t* __restrict__ stamp_idx) {
    pdl_wait();
    clear_stamps_kernel_body(S, c, stamp_idx, grid_blk());
}

// The sweep line through voxel idx for light along `axis` (the numbering the
// sweeps use: x rows by y + ny z, y columns by x + nx z, z columns by x + nx y).
__device__ __forceinline__ int64_t irr_line(const GridDev& I, int axis, int64_t idx) {
    const int64_t plane = (int64_t)I.nx * I.ny;
    if (axis == 0) return idx / I.nx;
    if (axis == 1) return idx % I.nx + (int64_t)I.nx * (idx / plane);
    return idx % plane;
}

// occlusion_stamp_kernel (emission.cu:17-27). The deposit words are zero
// before it (cleared by the previous emission stage) and every stamp is
// positive, so exactly one cell per stamped voxel sees zero come back from its
// add: that cell owns the voxel. Owners alone record the voxel (stamp_idx;
// other cells record -1), mark its line and set its bit, so the next emission
// stage clears each voxel once and the occlusion factor of each is computed
// once, not once per cell (a cluster core holds dozens of cells per voxel).
__device__ __forceinline__ void stamp_kernel_body(DevState* S, const Ctx& c, int32_t* stamp_idx, Blk blk) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    if (blk.x == 0 && threadIdx.x == 0) S->n_stamps = n;
    const GridDev I = c.g[AGB_FIELD_IRRADIANCE];
    AGB_FOR_CELLS_B(i, blk, n) {
        const uint32_t f = v.flags[i];
        int32_t rec = -1;
        if (f & AGB_FLAG_OCCUPIED) {
            const int64_t idx = grid_nearest(I, d2f(v.x[i]), d2f(v.y[i]), d2f(v.z[i]));
            const long long stamp = (f & AGB_FLAG_ALIVE) ? c.stamp_alive : c.stamp_dead;
            if (atomicAdd(&I.deposit[idx], (unsigned long long)stamp) == 0ull) {
                rec = (int32_t)idx;
                if (c.irr_marks) c.irr_marks[irr_line(I, c.light_axis, idx)] = 1;
                if (c.irr_stamp_bits) atomicOr(&c.irr_stamp_bits[idx >> 5], 1u << (idx & 31));
            }
        }
        stamp_idx[i] = rec;
    }
}

__global__ void stamp_kernel(DevState* S, Ctx c, int32_t* stamp_idx) {
    pdl_wait();
    stamp_kernel_body(S, c, stamp_idx, grid_blk());
}

// The FP64 divisions, out of line: only warps with a voxel outside the
// lookup table issue them.
__device__ __noinline__ double occlusion_fp64(unsigned long long dep, double scale, double face) {
    return occlusion_of((long long)dep, scale, face);
}

// column_transmittance (emission.cuh:43-47) of every stamped voxel, computed
// once per voxel by its owning cell, before the sweep (FP64 divisions in
// divergent sweep code would cost a whole warp's FP64 issue time per stamped
// voxel). Voxels holding one, two or three live cells or one dead cell take
// the factor from the world's table (the same bits); others divide.
__device__ __forceinline__ void occlusion_factor_kernel_body(DevState* S, const Ctx& c,
                                                             const int32_t* __restrict__ stamp_idx, double* factor,
                                                             Blk blk) {
    const int32_t n = S->n_stamps;
    const GridDev I = c.g[AGB_FIELD_IRRADIANCE];
    AGB_FOR_CELLS_B(i, blk, n) {
        const int32_t idx = stamp_idx[i];
        if (idx < 0) continue;
        const unsigned long long dep = I.deposit[idx];
        double f;
        if (dep == c.occl_dep[0]) f = c.occl_fac[0];
        else if (dep == c.occl_dep[1]) f = c.occl_fac[1];
        else if (dep == c.occl_dep[2]) f = c.occl_fac[2];
        else if (dep == c.occl_dep[3]) f = c.occl_fac[3];
        else f = occlusion_fp64(dep, I.scale, c.face_area);
        factor[idx] = f;
    }
}

__global__ void __launch_bounds__(256) occlusion_factor_kernel(DevState* S, Ctx c,
                                                               const int32_t* __restrict__ stamp_idx,
                                                               double* factor) {
    pdl_wait();
    occlusion_factor_kernel_body(S, c, stamp_idx, factor, grid_blk());
}

// Whether irradiance voxel idx was stamped this tick: its bit when the world
// keeps the bitmap, else its deposit word.
__device__ __forceinline__ bool stamped(const Ctx& c, const GridDev& I, int64_t idx) {
    if (c.irr_stamp_bits) return (__ldg(&c.irr_stamp_bits[idx >> 5]) >> (idx & 31)) & 1u;
    return __ldg(&I.deposit[idx]) != 0ull;
}

// sweep_kernel (emission.cu:37-53): one thread per line in sweep order. The
// FP64 transmittance recurrence runs only at stamped voxels (an empty voxel's
// factor is exactly 1), and the float output only changes there, so empty
// voxels cost one load and one store. The line is walked in chunks of
// SWEEP_PF voxels. The next chunk's stamp-bitmap words are loaded
// unconditionally (the step clamped to the line, so every address is in
// bounds) into registers while this chunk is written, and this chunk's
// occlusion factors are requested before its recurrence runs, so a chunk waits
// on at most one memory round trip. A bitmap word serves a warp's 32
// neighbouring lines at once along y and z. (The bitmap exists whenever the
// irradiance grid does.)
constexpr int SWEEP_PF = 16;

__device__ __forceinline__ void sweep_kernel_body(const Ctx& c, const double* __restrict__ factor, Blk blk) {
    const GridDev I = c.g[AGB_FIELD_IRRADIANCE];
    const int32_t nx = I.nx, ny = I.ny;
    const int64_t plane = (int64_t)nx * ny;
    const int axis = c.light_axis;
    const int32_t len = axis == 0 ? nx : (axis == 1 ? ny : I.nz);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? nx : plane);
    const int64_t lines = I.count / len;
    // Voxel of step s along a line: first + step * s.
    const int64_t step = c.light_sign > 0 ? stride : -stride;
    const uint32_t* __restrict__ bits = c.irr_stamp_bits;
    for (int64_t line = blk.x * (int64_t)blockDim.x + threadIdx.x; line < lines;
         line += (int64_t)blk.n * blockDim.x) {
        const uint8_t mark = c.irr_marks ? c.irr_marks[line] : 1;
        if (mark == 0) continue;                           // values already unshadowed
        if (c.irr_marks) c.irr_marks[line] = mark == 1 ? 2 : 0;
        int64_t base;
        if (axis == 0) base = line * nx;
        else if (axis == 1) base = (line % nx) + (line / nx) * plane;
        else base = line;
        const int64_t first = c.light_sign > 0 ? base : base + stride * (len - 1);
        double t = 1.0;
        float cur = fa(d2f(c.source_d * t), c.ambient_irr);
        uint32_t next[SWEEP_PF];                           // stamp-bitmap word of each step of the next chunk
#pragma unroll
        for (int u = 0; u < SWEEP_PF; ++u) next[u] = __ldg(&bits[(first + step * (u < len ? u : len - 1)) >> 5]);
        for (int32_t s0 = 0; s0 < len; s0 += SWEEP_PF) {
            bool raw[SWEEP_PF];
#pragma unroll
            for (int u = 0; u < SWEEP_PF; ++u) {
                const int32_t s = s0 + u;
                raw[u] = s < len && ((next[u] >> ((first + step * s) & 31)) & 1u) != 0u;
                const int32_t sn = s + SWEEP_PF;
                next[u] = __ldg(&bits[(first + step * (sn < len ? sn : len - 1)) >> 5]);
            }
            double fac[SWEEP_PF];
#pragma unroll
            for (int u = 0; u < SWEEP_PF; ++u) fac[u] = raw[u] ? __ldg(&factor[first + step * (s0 + u)]) : 1.0;
#pragma unroll
            for (int u = 0; u < SWEEP_PF; ++u) {
                const int32_t s = s0 + u;
                if (s >= len) break;
                I.value[first + step * s] = cur;
                if (raw[u]) {
                    t *= fac[u];
                    cur = fa(d2f(c.source_d * t), c.ambient_irr);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(128, 4) sweep_kernel(Ctx c, const double* __restrict__ factor) {
    pdl_wait();
    sweep_kernel_body(c, factor, grid_blk());
}

// 32 stamp bits of the row starting at voxel `rowbase`: bit m is voxel xa + m;
// voxels outside [0, len) read 0.
__device__ __forceinline__ uint32_t row_stamp_bits(const uint32_t* __restrict__ bits, int64_t nwords,
                                                   int64_t rowbase, int32_t xa, int32_t len) {
    const int32_t lo = xa < 0 ? 0 : xa;
    const int32_t hi = xa + 32 < len ? xa + 32 : len;
    if (hi <= lo) return 0u;
    const int64_t q = rowbase + lo;
    const int64_t wi = q >> 5;
    const int sh = (int)(q & 31);
    uint32_t v = __ldg(&bits[wi]) >> sh;
    if (sh && wi + 1 < nwords) v |= __ldg(&bits[wi + 1]) << (32 - sh);
    const int32_t n = hi - lo;
    if (n < 32) v &= (1u << n) - 1u;
    return v << (lo - xa);
}

// x-axis sweep (light along x): rows are contiguous in memory. A warp takes
// 32 rows and moves along them 32 voxels at a time. Each lane runs its own
// row's FP64 transmittance recurrence over the chunk's stamped voxels only,
// so the warp issues FP64 work as often as its busiest row has stamps in the
// chunk, not once per stamp of every row (FP64 issues at a small fraction of
// the FP32 rate). The value following each stamp goes to shared memory; the
// warp then writes the chunk row by row, 32 consecutive voxels per store: a
// voxel takes the value after its row's last stamp before it in sweep order,
// else the value the row entered the chunk with.
constexpr int SWEEP_ROW_WARPS = 8;       // sweep_rows_blocks and the batched launch assume 256 threads

__device__ __forceinline__ void sweep_rows_kernel_body(const Ctx& c, const double* __restrict__ factor, Blk blk) {
    __shared__ float after[SWEEP_ROW_WARPS][32][33];
    const GridDev I = c.g[AGB_FIELD_IRRADIANCE];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float (*buf)[33] = after[wib];
    const int32_t len = I.nx;
    const int64_t lines = I.count / len;
    const int64_t groups = (lines + 31) / 32;
    const int64_t nwords = (I.count + 31) / 32;
    const float entry = fa(d2f(c.source_d * 1.0), c.ambient_irr);
    for (int64_t g = (int64_t)blk.x * SWEEP_ROW_WARPS + wib; g < groups; g += (int64_t)blk.n * SWEEP_ROW_WARPS) {
        const int64_t row = g * 32 + lane;
        uint8_t mark = 0;
        if (row < lines) {
            mark = c.irr_marks ? c.irr_marks[row] : 1;
            if (c.irr_marks && mark) c.irr_marks[row] = mark == 1 ? 2 : 0;
        }
        const unsigned active = __ballot_sync(0xFFFFFFFFu, mark != 0);
        if (!active) continue;                              // every row already unshadowed
        const int64_t rowbase = row * len;
        double t = 1.0;
        float cur = entry;
        for (int32_t s0 = 0; s0 < len; s0 += 32) {
            uint32_t sb = 0u;
            if (mark) {
                sb = c.light_sign > 0 ? row_stamp_bits(c.irr_stamp_bits, nwords, rowbase, s0, len)
                                      : __brev(row_stamp_bits(c.irr_stamp_bits, nwords, rowbase, len - s0 - 32, len));
            }
            for (uint32_t m = sb; m; m &= m - 1u) {
                const int j = __ffs(m) - 1;
                const int32_t x = c.light_sign > 0 ? s0 + j : len - 1 - (s0 + j);
                t *= __ldg(&factor[rowbase + x]);
                buf[lane][j] = fa(d2f(c.source_d * t), c.ambient_irr);
            }
            __syncwarp();
            const int32_t s = s0 + lane;
            const int32_t x = c.light_sign > 0 ? s : len - 1 - s;
            const uint32_t before = (1u << lane) - 1u;
            for (unsigned a = active; a; a &= a - 1u) {
                const int r = __ffs(a) - 1;
                const uint32_t rb = __shfl_sync(0xFFFFFFFFu, sb, r) & before;
                const float rc = __shfl_sync(0xFFFFFFFFu, cur, r);
                const float v = rb ? buf[r][31 - __clz(rb)] : rc;
                if (s < len) I.value[(g * 32 + r) * len + x] = v;
            }
            if (sb) cur = buf[lane][31 - __clz(sb)];
            __syncwarp();
        }
    }
}

// The same sweep with one warp per row, 32 consecutive voxels per step; the
// FP64 recurrence walks the row's stamps in sweep order, broadcasting each
// factor. The warp issues the FP64 work once per stamp of its row, so this
// form wins only where rows are too few to give the 32-row tiles a wave
// (a single world's grid); batches take the tiles.
__device__ __forceinline__ void sweep_row_warps_kernel_body(const Ctx& c, const double* __restrict__ factor,
                                                            Blk blk) {
    const GridDev I = c.g[AGB_FIELD_IRRADIANCE];
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blk.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)blk.n * blockDim.x) >> 5;
    const int32_t len = I.nx;
    const int64_t lines = I.count / len;
    for (int64_t line = warp; line < lines; line += nwarps) {
        const uint8_t mark = c.irr_marks ? c.irr_marks[line] : 1;    // one byte, broadcast to the warp
        if (mark == 0) continue;                                    // values already unshadowed
        __syncwarp();
        if (c.irr_marks && lane == 0) c.irr_marks[line] = mark == 1 ? 2 : 0;
        const int64_t base = line * len;
        double t = 1.0;
        float cur = fa(d2f(c.source_d * t), c.ambient_irr);
        for (int32_t s0 = 0; s0 < len; s0 += 32) {
            const int32_t s = s0 + lane;
            const bool in = s < len;
            const int64_t idx = base + (c.light_sign > 0 ? s : (len - 1 - s));
            const bool raw = in && stamped(c, I, idx);
            unsigned mask = __ballot_sync(0xFFFFFFFFu, raw);
            float mine = cur;
            if (mask) {
                const double f = raw ? __ldg(&factor[idx]) : 1.0;
                while (mask) {
                    const int b = __ffs(mask) - 1;
                    mask &= mask - 1u;
                    t *= __shfl_sync(0xFFFFFFFFu, f, b);
                    cur = fa(d2f(c.source_d * t), c.ambient_irr);
                    if (lane > b) mine = cur;
                }
            }
            if (in) I.value[idx] = mine;
        }
    }
}

__global__ void __launch_bounds__(256) sweep_row_warps_kernel(Ctx c, const double* __restrict__ factor) {
    pdl_wait();
    sweep_row_warps_kernel_body(c, factor, grid_blk());
}

__global__ void __launch_bounds__(256) sweep_rows_kernel(Ctx c, const double* __restrict__ factor) {
    pdl_wait();
    sweep_rows_kernel_body(c, factor, grid_blk());
}

// disc_overlap_fraction / shadow_fraction in FP64 (emission.cuh:19-37): the
// decision path for near-degenerate geometry, rounded operation by operation
// as the reference writes it (no contraction: an FMA here would leave the
// rounding error of dx*dx in perp2 and turn an exact total shadow into 1e-8).
__device__ double shadow_fraction64(double dx, double dy, double dz, const Ctx& c) {
    const double along = __dadd_rn(__dadd_rn(__dmul_rn(dx, c.ldx), __dmul_rn(dy, c.ldy)), __dmul_rn(dz, c.ldz));
    if (along <= 0.0) return 0.0;
    const double len2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double perp2 = __dsub_rn(len2, __dmul_rn(along, along));
    const double p = perp2 > 0.0 ? sqrt(perp2) : 0.0;
    const double a = AGB_CELL_RADIUS;
    if (p <= 0.0) return 1.0;
    if (p >= 2.0 * a) return 0.0;
    const double x = __ddiv_rn(p, 2.0 * a);
    const double s = sqrt(__dsub_rn(1.0, __dmul_rn(x, x)));
    return __dmul_rn(2.0 / AGB_PI, __dsub_rn(acos(x), __dmul_rn(x, s)));
}

// feed_kernel (emission.cu:81-115), one thread per hash-sorted entry: warp
// lanes then share bucket neighbourhoods (broadcast loads of the candidate
// records) instead of each streaming its own list.
//
// With L > 1, L lanes share one cell's walk (small populations: more threads
// in flight per cell); the shading product is combined across them and lane 0
// writes the cell.
// One candidate k, at offset (dx, dy, dz) from the feeding cell (FP64
// position px, py, pz), against that cell's open fraction.
__device__ __forceinline__ void shade_candidate(const SoA& v, const Ctx& c, const HashDev& h, int32_t k, float dx,
                                                float dy, float dz, double px, double py, double pz, float& open,
                                                int32_t& refined) {
    const float two_a = (float)AGB_CELL_DIAMETER;
    const float a_f = (float)AGB_CELL_RADIUS;
    // Products and sums rounded explicitly: every kernel that inlines this
    // (per world or batched) forms the same bits.
    const float along = __fmaf_rn(dz, c.lz, __fmaf_rn(dy, c.ly, __fmul_rn(dx, c.lx)));
    // Geometry first (cheap, rejects most candidates); FP64 only near the
    // thresholds; the neighbour's flags only for real shadowers.
    if (along < -1e-6f * two_a) return;
    const float qx = __fmaf_rn(-along, c.lx, dx), qy = __fmaf_rn(-along, c.ly, dy), qz = __fmaf_rn(-along, c.lz, dz);
    const float perp = sqrtf(__fmaf_rn(qz, qz, __fmaf_rn(qy, qy, __fmul_rn(qx, qx))));
    if (along > 1e-6f * two_a && perp >= two_a * (1.0f + 1e-6f)) return;
    const int32_t j = (int32_t)__ldg(&h.vals_sorted[k]);
    if (!(v.flags[j] & AGB_FLAG_ALIVE)) return;   // current flags: thermal may have starved j
    if (along > 1e-6f * two_a && perp > 1e-2f * two_a && perp < two_a * (1.0f - 1e-6f)) {
        const float x = perp / (2.0f * a_f);
        const float frac = __fmul_rn(0.63661977f, __fmaf_rn(-x, sqrtf(__fmaf_rn(-x, x, 1.0f)), acosf(x)));
        open *= (1.0f - frac);
        return;
    }
    ++refined;   // both positions are this tick's (feeding moves nothing)
    const double fr = shadow_fraction64(__dsub_rn(px, v.x[j]), __dsub_rn(py, v.y[j]), __dsub_rn(pz, v.z[j]), c);
    open *= (float)(1.0 - fr);
}

// Under axis-aligned light every cell of the next bucket layer downstream has
// `along` < 0 (it sits in this cell's shadow-free half-space) and leaves
// `open` unchanged; a shading-only walk skips that layer when this cell is
// clear of its downstream bucket face by more than the FP32 offsets' error,
// so the product is unchanged.
__device__ __forceinline__ void shade_skip(const Ctx& c, const HashDev& h, const float4& me, int& skip_axis,
                                           int& skip_side) {
    skip_axis = -1;
    skip_side = 0;
    if (c.light_axis_exact >= 0) {
        const float off = c.light_axis_exact == 0 ? me.x : (c.light_axis_exact == 1 ? me.y : me.z);
        const float face = c.light_sign > 0 ? h.cellf - off : off;
        if (face > 4.0e-6f * h.cellf) { skip_axis = c.light_axis_exact; skip_side = c.light_sign; }
    }
}

// Directional irradiance at cell i before occlusion.
__device__ __forceinline__ float feed_directional(const Ctx& c, double px, double py, double pz) {
    const GridDev& I = c.g[AGB_FIELD_IRRADIANCE];
    const float d = fs(grid_sample(I, I.value, d2f(px), d2f(py), d2f(pz)), c.ambient_irr);
    return d < 0.0f ? 0.0f : d;
}

// Feeding's writes for cell i: irradiance and the energy gained.
__device__ __forceinline__ void feed_finish(const SoA& v, const Ctx& c, const TickParams& p, int32_t i,
                                            float directional) {
    v.irradiance[i] = directional;
    const float gained = __fmul_rn(__fmaf_rn(directional, (float)AGB_CELL_CROSS_SECTION,
                                             __fmul_rn(c.ambient_irr, (float)AGB_CELL_SURFACE_AREA)),
                                   p.dtf);
    double e = v.energy[i] + f2d(gained);
    if (dkey(e) > dkey(AGB_CELL_ENERGY_MAX)) e = AGB_CELL_ENERGY_MAX;
    v.energy[i] = e;
}

template <int L>
__device__ __forceinline__ void feed_cell(DevState* S, const SoA& v, const Ctx& c, const TickParams& p,
                                          int32_t ks, int32_t i, int lane, unsigned gm) {
    const HashDev h = c.h;
    const double px = v.x[i], py = v.y[i], pz = v.z[i];
    float directional = feed_directional(c, px, py, pz);
    // A cell in exact darkness stays dark whatever shades it: skip the walk
    // (directional * open is 0 for any open in [0, 1]).
    if (c.occlusion_exact && directional > 0.0f) {
        const float4 me = h.rec[ks];
        int32_t gx, gy, gz;
        unpack_bucket(me.w, gx, gy, gz);
        float open = 1.0f;
        int32_t refined = 0;
        int skip_axis, skip_side;
        shade_skip(c, h, me, skip_axis, skip_side);
        walk_neighbours<L>(h, gx, gy, gz, [&](int32_t k, const float4& rk, float cy, float cz) {
            if (k == ks) return;
            float dx, dy, dz;
            rec_delta(h, me, gx, rk, cy, cz, dx, dy, dz);
            shade_candidate(v, c, h, k, dx, dy, dz, px, py, pz, open, refined);
        }, skip_axis, skip_side, lane);
        if (L > 1) {
            open = group_prod<L>(open, gm);
            refined = group_isum<L>(refined, gm);
        }
        if (refined && lane == 0) atomicAdd(&S->n_shadow_refine, refined);
        directional *= open;
    }
    if (lane == 0) feed_finish(v, c, p, i, directional);
}

template <int L>
__global__ void __launch_bounds__(256) feed_kernel(DevState* S, Ctx c, TickParams p) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->hash_count;
    const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = t & (L - 1);
    const unsigned gm = group_mask<L>();
    for (int32_t ks = t / L; ks < n; ks += (int32_t)(gridDim.x * blockDim.x) / L) {
        const int32_t i = (int32_t)c.h.vals_sorted[ks];
        const uint32_t f = v.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        feed_cell<L>(S, v, c, p, ks, i, lane, gm);
    }
}

// ---------------------------------------------------------------------------
// Motion (src/sim/integrator.cu:20-150; src/sim/integrator.cuh:29-254)
// ---------------------------------------------------------------------------

// g(x) = 2x - 3 + 4e^-x - e^-2x (ou_position_shape, integrator.cuh:80-91) in
// FP32 without cancellation: Taylor series (terms to x^12) below 0.5, and
// 2(x + expm1(-x)) - expm1(-x)^2 above.
__device__ __forceinline__ float ou_shape_f(float x) {
    if (x < 0.5f) {
        float s = -4092.0f / 479001600.0f;
        s = 2044.0f / 39916800.0f + x * s;
        s = -1020.0f / 3628800.0f + x * s;
        s = 508.0f / 362880.0f + x * s;
        s = -252.0f / 40320.0f + x * s;
        s = 124.0f / 5040.0f + x * s;
        s = -1.0f / 12.0f + x * s;
        s = 7.0f / 30.0f + x * s;
        s = -0.5f + x * s;
        s = 2.0f / 3.0f + x * s;
        return x * x * x * s;
    }
    const float em = expm1f(-x);
    return __fmaf_rn(-em, em, __fmul_rn(2.0f, x + em));
}

// One axis of the joint OU propagator (ou_advance_axis, integrator.cuh:128-154):
// returns the position increment; updates the velocity.
__device__ __forceinline__ float ou_axis(float& vel, float force, float gamma, float dtf, float ome,
                                         float inv_beta, bool noise, float s_rr, float a, float b,
                                         float s_vv, float z1, float z2) {
    const float v_term = force / gamma;
    float dpos = __fmaf_rn(v_term, dtf, __fmul_rn(__fmul_rn(vel - v_term, ome), inv_beta));
    float nvel = __fmaf_rn(v_term - vel, ome, vel);
    if (noise && s_rr > 0.0f) {
        dpos = __fmaf_rn(s_rr, z1, dpos);
        nvel = __fadd_rn(nvel, __fmaf_rn(a, z1, __fmul_rn(b, z2)));
    } else if (noise) {
        nvel = __fmaf_rn(s_vv, z2, nvel);
    }
    vel = nvel;
    return dpos;
}

// apply_boundary_axis (integrator.cuh:233-254) on FP64 state with integer compares.
__device__ __forceinline__ bool boundary_axis(double& pos, float& vel, const Ctx& c, int ax, int mode) {
    const unsigned long long k = dkey(pos);
    if (k >= c.lo_key[ax] && k <= c.hi_key[ax]) return true;
    if (mode == AGB_WALL_PERIODIC) {
        // Bounded: a non-finite position must not spin forever.
        const double span = 2.0 * c.half[ax];
        for (int k = 0; k < 64 && pos < -c.half[ax]; ++k) pos += span;
        for (int k = 0; k < 64 && pos > c.half[ax]; ++k) pos -= span;
        return true;
    }
    if (mode == AGB_WALL_ABSORBING) return false;
    pos = (k < c.lo_key[ax]) ? c.lo[ax] : c.hi[ax];
    vel = 0.0f;
    return true;
}

// forces_kernel (integrator.cu:40-76), one thread per hash-sorted entry.
// With L > 1, L lanes share one cell's contact walk; their partial sums are
// combined and lane 0 writes the cell.
// One candidate k, at offset (dx, dy, dz) from cell i, against i's contact
// force (contact_force, integrator.cuh:200-219).
__device__ __forceinline__ void contact_candidate(const SoA& v, const HashDev& h, const TickParams& p, int32_t k,
                                                  int32_t i, float dx, float dy, float dz, float& Cx, float& Cy,
                                                  float& Cz, int32_t& refined) {
    const float two_a = (float)AGB_CELL_DIAMETER;
    const float thr = two_a * two_a;
    const double two_a64 = AGB_CELL_DIAMETER;
    const float r2s = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    if (r2s >= thr * (1.0f + 1e-5f)) return;                     // clear of contact
    if (r2s <= thr * (1.0f - 1e-5f) && r2s > 1e-12f * thr) {     // in contact
        const float r = sqrtf(r2s);
        const float s = p.k_contact * (two_a - r) / r;
        Cx = __fmaf_rn(dx, s, Cx); Cy = __fmaf_rn(dy, s, Cy); Cz = __fmaf_rn(dz, s, Cz);
        return;
    }
    ++refined;   // settle in FP64 from the pre-step positions (integrator.cuh:210-219)
    const int32_t j = (int32_t)__ldg(&h.vals_sorted[k]);
    const double ddx = __dsub_rn(v.x[i], v.x[j]), ddy = __dsub_rn(v.y[i], v.y[j]), ddz = __dsub_rn(v.z[i], v.z[j]);
    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
    if (rr >= two_a64 * two_a64 || rr <= 0.0) return;
    const double r = sqrt(rr);
    const double s = __ddiv_rn(__dmul_rn(p.k_contact64, __dsub_rn(two_a64, r)), r);
    Cx += (float)__dmul_rn(ddx, s); Cy += (float)__dmul_rn(ddy, s); Cz += (float)__dmul_rn(ddz, s);
}

// field_sample_kernel (integrator.cu:20-30) for cell i: sorted order makes
// neighbouring threads sample neighbouring voxels.
__device__ __forceinline__ void sample_fields(const SoA& v, const Ctx& c, int32_t i) {
    const GridDev& T = c.g[AGB_FIELD_TEMPERATURE];
    const GridDev& C2 = c.g[AGB_FIELD_CO2];
    const GridDev& N2 = c.g[AGB_FIELD_N2];
    const float xf = d2f(v.x[i]), yf = d2f(v.y[i]), zf = d2f(v.z[i]);
    if (T.enabled) v.t_local[i] = grid_sample(T, T.value, xf, yf, zf);
    if (C2.enabled) v.co2_local[i] = grid_sample(C2, C2.value, xf, yf, zf);
    if (N2.enabled) v.n2_local[i] = grid_sample(N2, N2.value, xf, yf, zf);
}

// Net force on cell i (integrator.cu:40-76): buoyancy, photon thrust, the
// summed contacts (Cx, Cy, Cz; added only when contacts are on) and the trap.
__device__ __forceinline__ void forces_finish(const SoA& v, const Ctx& c, const TickParams& p, int32_t i, float Cx,
                                              float Cy, float Cz, float* fx_out, float* fy_out, float* fz_out) {
    const uint32_t flags = v.flags[i];
    const float mass = __fmaf_rn(d2f(v.energy[i]), (float)(1.0 / (AGB_C_LIGHT * AGB_C_LIGHT)), d2f(v.biomass[i]));
    const bool alive = (flags & AGB_FLAG_ALIVE) != 0u;
    const float wgt = -(mass - (float)(AGB_WATER_DENSITY * AGB_CELL_VOLUME)) * (float)AGB_G_ACCEL;
    float Fx = 0.0f, Fy = 0.0f, Fz = 0.0f;
    if (c.gravity_axis == AGB_GRAVITY_Y) Fy += wgt; else Fz += wgt;
    const float thrust = alive ? v.emit_power[i] * (float)(1.0 / AGB_C_LIGHT) : 0.0f;
    if (thrust != 0.0f) {
        Fx = __fmaf_rn(-v.dir_x[i], thrust, Fx);
        Fy = __fmaf_rn(-v.dir_y[i], thrust, Fy);
        Fz = __fmaf_rn(-v.dir_z[i], thrust, Fz);
    }
    if (c.contact_enabled) { Fx += Cx; Fy += Cy; Fz += Cz; }
    if (i == c.trap_slot) {                                      // trap_force (integrator.cuh:195-197)
        Fx = __fmaf_rn(p.k_trap, (float)(c.trap_x - v.x[i]), Fx);
        Fy = __fmaf_rn(p.k_trap, (float)(c.trap_y - v.y[i]), Fy);
    }
    fx_out[i] = Fx; fy_out[i] = Fy; fz_out[i] = Fz;
}

template <int L>
__device__ __forceinline__ void forces_cell(DevState* S, const SoA& v, const Ctx& c, const TickParams& p,
                                            int32_t ks, int32_t i, int lane, unsigned gm, float* fx_out,
                                            float* fy_out, float* fz_out) {
    const HashDev h = c.h;
    float Cx = 0.0f, Cy = 0.0f, Cz = 0.0f;
    if (c.contact_enabled) {
        const float4 me = h.rec[ks];
        int32_t gx, gy, gz;
        unpack_bucket(me.w, gx, gy, gz);
        int32_t refined = 0;
        walk_neighbours<L>(h, gx, gy, gz, [&](int32_t k, const float4& rk, float cy, float cz) {
            if (k == ks) return;                                    // bucket members are occupied
            float dx, dy, dz;
            rec_delta(h, me, gx, rk, cy, cz, dx, dy, dz);
            contact_candidate(v, h, p, k, i, dx, dy, dz, Cx, Cy, Cz, refined);
        }, -1, 0, lane);
        if (L > 1) {
            Cx = group_sum<L>(Cx, gm);
            Cy = group_sum<L>(Cy, gm);
            Cz = group_sum<L>(Cz, gm);
            refined = group_isum<L>(refined, gm);
        }
        if (refined && lane == 0) atomicAdd(&S->n_contact_refine, refined);
    }
    if (lane != 0) return;
    sample_fields(v, c, i);
    forces_finish(v, c, p, i, Cx, Cy, Cz, fx_out, fy_out, fz_out);
}

template <int L>
__global__ void __launch_bounds__(256) forces_kernel(DevState* S, Ctx c, TickParams p, float* fx_out,
                                                     float* fy_out, float* fz_out) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->hash_count;
    const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = t & (L - 1);
    const unsigned gm = group_mask<L>();
    for (int32_t ks = t / L; ks < n; ks += (int32_t)(gridDim.x * blockDim.x) / L) {
        const int32_t i = (int32_t)c.h.vals_sorted[ks];
        if (c.h.keys_sorted[ks] >= (uint32_t)c.h.buckets) {      // unoccupied slot (sentinel key)
            if (lane == 0) { fx_out[i] = 0.0f; fy_out[i] = 0.0f; fz_out[i] = 0.0f; }
            continue;
        }
        forces_cell<L>(S, v, c, p, ks, i, lane, gm, fx_out, fy_out, fz_out);
    }
}

// integrate_kernel (integrator.cu:79-150), slot order (coalesced state access).
// With `demand` set, the lifecycle's demand pass (demand_kernel,
// lifecycle.cu:41-57) runs here on each live cell at its new position.
__device__ __forceinline__ void integrate_kernel_body(DevState* S, const Ctx& c, const TickParams& p,
                                                      const float* __restrict__ fx_in,
                                                      const float* __restrict__ fy_in,
                                                      const float* __restrict__ fz_in, const GridDev& co2,
                                                      unsigned long long* demand, double gv, double* want,
                                                      int32_t* vox, Blk blk) {
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS_B(i, blk, n) {
        const uint32_t flags = v.flags[i];
        if (!(flags & AGB_FLAG_OCCUPIED)) continue;
        double px = v.x[i], py = v.y[i], pz = v.z[i];
        const float t_local = v.t_local[i];       // sampled by forces_kernel this tick
        const float Fx = fx_in[i], Fy = fy_in[i], Fz = fz_in[i];
        const float mass = __fmaf_rn(d2f(v.energy[i]), (float)(1.0 / (AGB_C_LIGHT * AGB_C_LIGHT)), d2f(v.biomass[i]));
        // integrate_kernel (integrator.cu:79-150)
        const bool awake = (flags & AGB_FLAG_AWAKE) != 0u;
        const float t_drag = awake ? (float)AGB_CELL_TEMP_SETPOINT : t_local;
        float gamma = (float)(6.0 * AGB_PI * AGB_CELL_RADIUS * AGB_VF_A) *
                      expf((float)AGB_VF_B / (t_drag - (float)AGB_VF_C));
        if (flags & AGB_FLAG_STUCK) gamma *= (float)AGB_WALL_STUCK_DRAG_MULT;
        // ou_coefficients (integrator.cuh:103-121)
        const float beta = gamma / mass;
        const float x = beta * p.dtf;
        const float ome = -expm1f(-x);
        const float inv_beta = 1.0f / beta;
        const float kTm = (float)AGB_K_BOLTZ * t_drag / mass;
        const float var_vv = kTm * (-expm1f(-2.0f * x));
        const float var_rr = kTm * inv_beta * inv_beta * ou_shape_f(x);
        const float s_vv = sqrtf(var_vv > 0.0f ? var_vv : 0.0f);
        const float s_rr = sqrtf(var_rr > 0.0f ? var_rr : 0.0f);
        const float s_rv = kTm * inv_beta * ome * ome;
        float a = 0.0f, b = 0.0f;
        if (s_rr > 0.0f) {
            a = s_rv / s_rr;
            const float b2 = __fmaf_rn(s_vv, s_vv, -__fmul_rn(a, a));
            b = sqrtf(b2 > 0.0f ? b2 : 0.0f);
        }
        Pcg rng{v.rng_state[i], cell_stream_inc(v.id[i])};
        float z1, z2, z3, z4, z5, z6;
        gaussian_pair_f(rng, z1, z2);
        gaussian_pair_f(rng, z3, z4);
        gaussian_pair_f(rng, z5, z6);
        float ux = d2f(v.vx[i]), uy = d2f(v.vy[i]), uz = d2f(v.vz[i]);
        const bool noise = c.thermal_noise != 0;
        const float dpx = ou_axis(ux, Fx, gamma, p.dtf, ome, inv_beta, noise, s_rr, a, b, s_vv, z1, z2);
        const float dpy = ou_axis(uy, Fy, gamma, p.dtf, ome, inv_beta, noise, s_rr, a, b, s_vv, z3, z4);
        const float dpz = ou_axis(uz, Fz, gamma, p.dtf, ome, inv_beta, noise, s_rr, a, b, s_vv, z5, z6);
        px += f2d(dpx);
        py += f2d(dpy);
        pz += f2d(dpz);
        bool kept = boundary_axis(px, ux, c, 0, c.boundary_x);
        kept = boundary_axis(py, uy, c, 1, c.boundary_y) && kept;
        const unsigned long long zb = (unsigned long long)__double_as_longlong(pz);
        boundary_axis(pz, uz, c, 2, AGB_WALL_REFLECTING);
        const bool touched = (unsigned long long)__double_as_longlong(pz) != zb;
        uint32_t nf = flags;
        if (c.adhesion_enabled) {
            if (touched && !(flags & AGB_FLAG_STUCK)) {
                if (uniform53(rng) < c.stick_bits) nf |= AGB_FLAG_STUCK;
            } else if (flags & AGB_FLAG_STUCK) {
                const float away = (pz < 0.0) ? Fz : -Fz;
                if (away > (float)AGB_WALL_RELEASE_FORCE) nf &= ~AGB_FLAG_STUCK;
            }
        }
        v.rng_state[i] = rng.state;
        if (!kept) {
            nf &= ~AGB_FLAG_ALIVE;
            v.death_cause[i] = AGB_DEATH_CULLED;
            v.emit_power[i] = 0.0f;
        }
        v.flags[i] = nf;
        v.x[i] = px; v.y[i] = py; v.z[i] = pz;
        v.vx[i] = f2d(ux); v.vy[i] = f2d(uy); v.vz[i] = f2d(uz);
        v.age_s[i] = v.age_s[i] + p.dtf;
        if (demand) {
            if (nf & AGB_FLAG_ALIVE) co2_demand_cell(co2, p, d2f(px), d2f(py), d2f(pz), demand, gv, want, vox, i);
            else if (vox) vox[i] = -1;
        }
    }
}

__global__ void __launch_bounds__(256) integrate_kernel(DevState* S, Ctx c, TickParams p,
                                                        const float* __restrict__ fx_in,
                                                        const float* __restrict__ fy_in,
                                                        const float* __restrict__ fz_in, GridDev co2,
                                                        unsigned long long* demand, double gv, double* want,
                                                        int32_t* vox) {
    pdl_wait();
    integrate_kernel_body(S, c, p, fx_in, fy_in, fz_in, co2, demand, gv, want, vox, grid_blk());
}

// ---------------------------------------------------------------------------
// Taxis (src/sim/taxis.cu:13-77 with src/sim/taxis.cuh:31-143). Per cell, in
// slot order. FP64 as the reference, every product and sum explicitly rounded
// (no contraction), so integer outcomes (state, tumble, RNG draws) and the
// stored floats follow the reference; log/sin/cos are CUDA's (within an ulp
// or two of the host's).
// ---------------------------------------------------------------------------
struct V3 { double x, y, z; };
__device__ __forceinline__ double dot3(V3 a, V3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 scale3(V3 a, double s) { return V3{__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return V3{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
              __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ V3 normalize3(V3 a) {                 // vec.cuh:34-37
    const double l = __dsqrt_rn(dot3(a, a));
    return l > 0.0 ? scale3(a, __drcp_rn(l)) : V3{0.0, 0.0, 1.0};
}
__device__ V3 taxis_tumble(V3 heading, Pcg& rng) {               // taxis.cuh:104-118
    double theta = __dmul_rn(-AGB_TAXIS_TUMBLE_ANGLE_MEAN, log(__dsub_rn(1.0, uniform01d(rng))));
    if (theta > AGB_PI) theta = AGB_PI;
    const double azimuth = __dmul_rn(AGB_TWO_PI, uniform01d(rng));
    const V3 h = normalize3(heading);
    const double ax = fabs(h.x), ay = fabs(h.y), az = fabs(h.z);  // any_perpendicular, taxis.cuh:86-92
    const V3 axis = (ax <= ay && ax <= az) ? V3{1.0, 0.0, 0.0} : (ay <= az) ? V3{0.0, 1.0, 0.0} : V3{0.0, 0.0, 1.0};
    const V3 u = normalize3(cross3(h, axis));
    const V3 w = cross3(h, u);
    double sa, ca, st, ct;
    sincos(azimuth, &sa, &ca);
    sincos(theta, &st, &ct);
    const V3 perp = add3(scale3(u, ca), scale3(w, sa));           // rotate_by, taxis.cuh:95-100
    return normalize3(add3(scale3(h, ct), scale3(perp, st)));
}

__device__ __forceinline__ void taxis_cell(const SoA& v, const TickParams& p, int32_t i) {
    const uint32_t f = v.flags[i];
    if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) return;
    if (!(f & AGB_FLAG_AWAKE)) {                               // dormant: inert, no emission
        v.emit_power[i] = 0.0f;
        return;
    }
    const double irr = (double)v.irradiance[i];
    const double co2 = (double)v.co2_local[i];
    const double energy = v.energy[i];
    const double charge = div_known(energy, AGB_CELL_ENERGY_MAX, 1.0 / AGB_CELL_ENERGY_MAX);
    const bool dark = irr < AGB_TAXIS_DARK_THRESHOLD, co2_here = co2 > 0.0;   // taxis.cuh:56-62
    int state = 0;                                             // 0 idle, 1 feed, 2 breed
    if (!(dark && !co2_here)) {
        if (!dark && charge < AGB_TAXIS_SEEK_FEED_BELOW) state = 1;
        else if (charge > AGB_TAXIS_SEEK_BREED_ABOVE && co2_here) state = 2;
    }
    if (state == 0) {                                          // no draws on the idle path
        v.emit_power[i] = 0.0f;
        v.run_timer[i] = 0.0f;
        v.taxis_memory[i] = 0.0f;
        return;
    }
    const double signal = state == 1 ? irr : co2;
    const double mem = (double)v.taxis_memory[i];
    const double delta = __dsub_rn(signal, mem);
    v.taxis_memory[i] = (float)__dadd_rn(mem, __dmul_rn(p.taxis_alpha, __dsub_rn(signal, mem)));
    V3 heading{-(double)v.dir_x[i], -(double)v.dir_y[i], -(double)v.dir_z[i]};
    double run = __dadd_rn((double)v.run_timer[i], p.dt);
    if (delta <= 0.0 || run >= AGB_TAXIS_RUN_MAX) {            // taxis_should_tumble
        Pcg rng{v.rng_state[i], cell_stream_inc(v.id[i])};
        heading = taxis_tumble(heading, rng);
        v.rng_state[i] = rng.state;
        run = 0.0;
    }
    v.run_timer[i] = (float)run;
    const V3 nh = normalize3(heading);                         // taxis_emit_dir = -normalize(heading)
    v.dir_x[i] = (float)(-nh.x);
    v.dir_y[i] = (float)(-nh.y);
    v.dir_z[i] = (float)(-nh.z);
    double pw = 0.0;                                           // taxis_emit_power, taxis.cuh:136-141
    if (energy > 0.0) {
        const double avail = p.dt > 0.0 ? div_known(energy, p.dt, p.dt_inv) : 0.0;
        pw = p.max_emit_power < avail ? p.max_emit_power : avail;
    }
    v.emit_power[i] = (float)pw;
    v.energy[i] = __dsub_rn(energy, __dmul_rn(pw, p.dt));
}

// flash_kernel (src/sim/flash.cu:31-56): every awake live cell discharges
// power * dt of its store (no more than it holds), with no free-cell thrust;
// the photon impulse (along -z) and the discharged energy go to the audit in
// fixed point, summed per warp first (integer sums: any order gives the same
// words).
__global__ void __launch_bounds__(256) flash_kernel(DevState* S, double dt, double power,
                                                    unsigned long long* accum) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->count;
    const double de0 = __dmul_rn(power, dt);
    for (int32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int32_t i = base + threadIdx.x;
        long long imp_q = 0, e_q = 0;
        if (i < n) {
            const uint32_t f = v.flags[i];
            if ((f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE) && (f & AGB_FLAG_AWAKE)) {
                const double e = v.energy[i];
                v.emit_power[i] = 0.0f;
                if (!(e <= 0.0)) {
                    const double de = de0 > e ? e : de0;
                    v.energy[i] = __dsub_rn(e, de);
                    const double imp = __ddiv_rn(de, AGB_C_LIGHT);
                    imp_q = llround(__dmul_rn(-imp, AGB_FLASH_IMPULSE_SCALE));
                    e_q = llround(__dmul_rn(de, AGB_FLASH_ENERGY_SCALE));
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            imp_q += __shfl_down_sync(0xFFFFFFFFu, imp_q, o);
            e_q += __shfl_down_sync(0xFFFFFFFFu, e_q, o);
        }
        if ((threadIdx.x & 31) == 0 && (imp_q | e_q)) {
            atomicAdd(&accum[2], (unsigned long long)imp_q);
            atomicAdd(&accum[3], (unsigned long long)e_q);
        }
    }
}

__global__ void __launch_bounds__(256) taxis_kernel(DevState* S, Ctx c, TickParams p) {
    pdl_wait();
    const SoA v = S->cur;
    const int32_t n = S->count;
    AGB_FOR_CELLS(i, n) taxis_cell(v, p, i);
}

// The per-cell middle of the tick in one pass over the hash-sorted entries:
// feeding (emission.cu:81-115), taxis (taxis.cu:13-85) and field sample +
// forces (integrator.cu:20-76) for each cell in turn, with ONE neighbour walk
// that applies both the shading and the contact test to every candidate.
// Each stage reads and writes only its own cell's state, apart from
// neighbours' positions and flags, which none of them changes, and each lane
// visits candidates in the order of the separate walks, so every cell gets
// the values the three separate passes give it. (A shading-only walk may skip
// the downstream layer under axis-aligned light; the shared walk visits it,
// and its candidates leave `open` unchanged.) `feed` / `taxis` select the
// stages this tick runs; with L > 1 the group shares the walk and lane 0
// finishes the cell.
template <int L>
__device__ __forceinline__ void cell_step_kernel_body(DevState* S, const Ctx& c, const TickParams& p, int feed,
                                                      int taxis, float* fx_out, float* fy_out, float* fz_out,
                                                      Blk blk) {
    const SoA v = S->cur;
    const HashDev h = c.h;
    const int32_t n = S->hash_count;
    const int32_t t = blk.x * blockDim.x + threadIdx.x;
    const int lane = t & (L - 1);
    const unsigned gm = group_mask<L>();
    const bool contact = c.contact_enabled != 0;
    for (int32_t ks = t / L; ks < n; ks += (int32_t)(blk.n * blockDim.x) / L) {
        const int32_t i = (int32_t)h.vals_sorted[ks];
        if (h.keys_sorted[ks] >= (uint32_t)h.buckets) {          // unoccupied slot (sentinel key)
            if (lane == 0) { fx_out[i] = 0.0f; fy_out[i] = 0.0f; fz_out[i] = 0.0f; }
            continue;
        }
        const uint32_t f = v.flags[i];
        const bool fd = feed && (f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE);
        const double px = v.x[i], py = v.y[i], pz = v.z[i];
        float directional = fd ? feed_directional(c, px, py, pz) : 0.0f;
        // A cell in exact darkness needs no shading test (directional * open
        // is 0 for any open in [0, 1]); its contacts are still walked.
        const bool shade = fd && c.occlusion_exact && directional > 0.0f;
        float open = 1.0f, Cx = 0.0f, Cy = 0.0f, Cz = 0.0f;
        int32_t rs = 0, rc = 0;
        if (shade || contact) {
            const float4 me = h.rec[ks];
            int32_t gx, gy, gz;
            unpack_bucket(me.w, gx, gy, gz);
            int skip_axis = -1, skip_side = 0;
            if (!contact) shade_skip(c, h, me, skip_axis, skip_side);
            walk_neighbours<L>(h, gx, gy, gz, [&](int32_t k, const float4& rk, float cy, float cz) {
                if (k == ks) return;
                float dx, dy, dz;
                rec_delta(h, me, gx, rk, cy, cz, dx, dy, dz);
                if (shade) shade_candidate(v, c, h, k, dx, dy, dz, px, py, pz, open, rs);
                if (contact) contact_candidate(v, h, p, k, i, dx, dy, dz, Cx, Cy, Cz, rc);
            }, skip_axis, skip_side, lane);
            if (L > 1) {
                if (shade) {
                    open = group_prod<L>(open, gm);
                    rs = group_isum<L>(rs, gm);
                }
                if (contact) {
                    Cx = group_sum<L>(Cx, gm);
                    Cy = group_sum<L>(Cy, gm);
                    Cz = group_sum<L>(Cz, gm);
                    rc = group_isum<L>(rc, gm);
                }
            }
        }
        if (lane != 0) continue;
        if (rs) atomicAdd(&S->n_shadow_refine, rs);
        if (rc) atomicAdd(&S->n_contact_refine, rc);
        if (fd) {
            if (shade) directional *= open;
            feed_finish(v, c, p, i, directional);
        }
        if (taxis) taxis_cell(v, p, i);
        sample_fields(v, c, i);
        forces_finish(v, c, p, i, Cx, Cy, Cz, fx_out, fy_out, fz_out);
    }
}

template <int L>
__global__ void __launch_bounds__(256) cell_step_kernel(DevState* S, Ctx c, TickParams p, int feed, int taxis,
                                                        float* fx_out, float* fy_out, float* fz_out) {
    pdl_wait();
    cell_step_kernel_body<L>(S, c, p, feed, taxis, fx_out, fy_out, fz_out, grid_blk());
}

// ---------------------------------------------------------------------------
// Batched launches of the per-cell stages (agb_batch): one grid over many
// chambers, each block running the per-world body for its chamber.
// ---------------------------------------------------------------------------
AGB_BATCHED_MB(thermal_batch, 256, 4, thermal_kernel_body(a.S, a.c, a.p, a.arg != 0, blk))
AGB_BATCHED(clear_stamps_batch, 256, clear_stamps_kernel_body(a.S, a.c, a.stamp_idx, blk))
AGB_BATCHED(stamp_batch, 256, stamp_kernel_body(a.S, a.c, a.stamp_idx, blk))
AGB_BATCHED(occlusion_factor_batch, 256, occlusion_factor_kernel_body(a.S, a.c, a.stamp_idx, a.factor, blk))
AGB_BATCHED(sweep_rows_batch, 256, sweep_rows_kernel_body(a.c, a.factor, blk))
AGB_BATCHED_MB(sweep_lines_batch, 128, 4, sweep_kernel_body(a.c, a.factor, blk))
AGB_BATCHED_MB(cell_step_batch, 256, 4,
            cell_step_kernel_body<1>(a.S, a.c, a.p, a.arg & 1, (a.arg >> 1) & 1, a.fx, a.fy, a.fz, blk))
AGB_BATCHED_MB(integrate_batch, 256, 4,
            integrate_kernel_body(a.S, a.c, a.p, a.fx, a.fy, a.fz, a.g, a.demand, a.gv, a.life.co2_want,
                                  a.life.co2_vox, blk))

}  // namespace

int32_t bstage_threads(BStage st) {
    switch (st) {
        case BStage::SweepLines: return 128;
        case BStage::Swap: return 32;
        default: return 256;
    }
}

void launch_batched(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, int32_t arg,
                    cudaStream_t s) {
    if (blocks <= 0) return;
    if (launch_batched_cells(st, tab, map, blocks, s)) return;
    if (launch_batched_grid(st, tab, map, blocks, s)) return;
    if (launch_batched_hash(st, tab, map, blocks, arg, s)) return;
    launch_batched_life(st, tab, map, blocks, arg, s);
}

bool launch_batched_cells(BStage st, const ChamberArgs* tab, const uint32_t* map, int32_t blocks, cudaStream_t s) {
    const unsigned g = (unsigned)blocks;
    switch (st) {
        case BStage::Thermal: launch_k(thermal_batch, g, 256, 0, s, tab, map); return true;
        case BStage::ClearStamps: launch_k(clear_stamps_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Stamp: launch_k(stamp_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Occlusion: launch_k(occlusion_factor_batch, g, 256, 0, s, tab, map); return true;
        case BStage::SweepRows: launch_k(sweep_rows_batch, g, 256, 0, s, tab, map); return true;
        case BStage::SweepLines: launch_k(sweep_lines_batch, g, 128, 0, s, tab, map); return true;
        case BStage::CellStep: launch_k(cell_step_batch, g, 256, 0, s, tab, map); return true;
        case BStage::Integrate: launch_k(integrate_batch, g, 256, 0, s, tab, map); return true;
        default: return false;
    }
}

void launch_flash(DevState* S, double dt, double power, unsigned long long* accum, int32_t blocks, cudaStream_t s) {
    launch_k(flash_kernel, blocks, 256, 0, s, S, dt, power, accum);
}

void launch_taxis(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, cudaStream_t s) {
    launch_k(taxis_kernel, blocks, 256, 0, s, S, c, p);
}

void launch_thermal(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, bool first, cudaStream_t s) {
    launch_k(thermal_kernel, blocks, 256, 0, s, S, c, p, first ? 1 : 0);
}
static int sm_count_of_device() {
    static int sms = 0;
    if (sms == 0) {
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

void launch_emission_prep(DevState* S, const Ctx& c, const TickParams& p, int32_t* stamp_idx, double* factor,
                          bool stamp, int32_t blocks, cudaStream_t s) {
    (void)p;
    launch_k(clear_stamps_kernel, blocks, 256, 0, s, S, c, stamp_idx);
    if (stamp) {
        launch_k(stamp_kernel, blocks, 256, 0, s, S, c, stamp_idx);
        launch_k(occlusion_factor_kernel, blocks, 256, 0, s, S, c, stamp_idx, factor);
    }
    const GridDev& I = c.g[AGB_FIELD_IRRADIANCE];
    const int32_t len = c.light_axis == 0 ? I.nx : (c.light_axis == 1 ? I.ny : I.nz);
    const int64_t lines = I.count / len;
    if (c.light_axis == 0) {
        // Tiles of 32 rows need rows for several waves; a single world's grid
        // rarely has them (a 128^3 grid has 16,384 rows, 64 tile blocks).
        if (lines >= 32 * 4 * SWEEP_ROW_WARPS * (int64_t)sm_count_of_device()) {
            launch_k(sweep_rows_kernel, (unsigned)sweep_rows_blocks(lines), 32 * SWEEP_ROW_WARPS, 0, s, c, factor);
        } else {
            const int64_t blocks = (lines * 32 + 255) / 256;
            launch_k(sweep_row_warps_kernel, (unsigned)(blocks < 65535 ? blocks : 65535), 256, 0, s, c, factor);
        }
    } else {
        launch_k(sweep_kernel, (unsigned)((lines + 127) / 128), 128, 0, s, c, factor);
    }
}
// Grid for a walk kernel with `lanes` threads per cell: `blocks` covers the
// population one thread per cell, so it grows by `lanes` (bounded).
static unsigned walk_blocks(int32_t blocks, int lanes) {
    const int64_t b = (int64_t)blocks * lanes;
    return (unsigned)(b < 65535 ? b : 65535);
}
void launch_feed(DevState* S, const Ctx& c, const TickParams& p, int32_t blocks, int lanes, cudaStream_t s) {
    const unsigned g = walk_blocks(blocks, lanes);
    switch (lanes) {
        case 8: launch_k(feed_kernel<8>, g, 256, 0, s, S, c, p); break;
        case 4: launch_k(feed_kernel<4>, g, 256, 0, s, S, c, p); break;
        case 2: launch_k(feed_kernel<2>, g, 256, 0, s, S, c, p); break;
        default: launch_k(feed_kernel<1>, blocks, 256, 0, s, S, c, p); break;
    }
}
void launch_emission(DevState* S, const Ctx& c, const TickParams& p, int32_t* stamp_idx, double* factor,
                     bool stamp, int32_t blocks, int lanes, cudaStream_t s) {
    launch_emission_prep(S, c, p, stamp_idx, factor, stamp, blocks, s);
    launch_feed(S, c, p, blocks, lanes, s);
}
void launch_cell_step(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                      int32_t blocks, int lanes, bool feed, bool taxis, cudaStream_t s) {
    const unsigned g = walk_blocks(blocks, lanes);
    const int fe = feed ? 1 : 0, tx = taxis ? 1 : 0;
    switch (lanes) {
        case 8: launch_k(cell_step_kernel<8>, g, 256, 0, s, S, c, p, fe, tx, fx, fy, fz); break;
        case 4: launch_k(cell_step_kernel<4>, g, 256, 0, s, S, c, p, fe, tx, fx, fy, fz); break;
        case 2: launch_k(cell_step_kernel<2>, g, 256, 0, s, S, c, p, fe, tx, fx, fy, fz); break;
        default: launch_k(cell_step_kernel<1>, blocks, 256, 0, s, S, c, p, fe, tx, fx, fy, fz); break;
    }
}
void launch_forces(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                   int32_t blocks, int lanes, cudaStream_t s) {
    const unsigned g = walk_blocks(blocks, lanes);
    switch (lanes) {
        case 8: launch_k(forces_kernel<8>, g, 256, 0, s, S, c, p, fx, fy, fz); break;
        case 4: launch_k(forces_kernel<4>, g, 256, 0, s, S, c, p, fx, fy, fz); break;
        case 2: launch_k(forces_kernel<2>, g, 256, 0, s, S, c, p, fx, fy, fz); break;
        default: launch_k(forces_kernel<1>, blocks, 256, 0, s, S, c, p, fx, fy, fz); break;
    }
}
void launch_integrate(DevState* S, const Ctx& c, const TickParams& p, const float* fx, const float* fy,
                      const float* fz, int32_t blocks, const GridDev& co2, unsigned long long* demand,
                      double gv, double* want, int32_t* vox, cudaStream_t s) {
    launch_k(integrate_kernel, blocks, 256, 0, s, S, c, p, fx, fy, fz, co2, demand, gv, want, vox);
}
void launch_motion(DevState* S, const Ctx& c, const TickParams& p, float* fx, float* fy, float* fz,
                   int32_t blocks, int lanes, cudaStream_t s) {
    launch_forces(S, c, p, fx, fy, fz, blocks, lanes, s);
    launch_integrate(S, c, p, fx, fy, fz, blocks, c.g[AGB_FIELD_CO2], nullptr, 0.0, nullptr, nullptr, s);
}

}  // namespace agb
