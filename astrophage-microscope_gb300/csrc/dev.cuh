// dev.cuh -- device-side types and helpers shared by every engine kernel.
//
// Precision policy (GB300: FP64 issues at ~1.6 op/clk/SM against ~112 for
// FP32, measured): contract state stays FP64 in memory, but per-cell math runs
// in FP32. FP64 is used only (a) to commit deltas into FP64 state, (b) in the
// rare events (division), and (c) to settle decisions whose FP32 estimate lies
// within its error bound of a threshold, so integer outcomes (hash keys,
// contact pairs, the exact-zero shadow set, wall contacts) equal the
// reference's FP64 decisions. Field arithmetic that the reference does in FP32
// uses explicitly rounded intrinsics in the reference's evaluation order, so
// fields match the reference bit for bit.
#pragma once

#include <cstdint>

#include "../../include/agb.h"
#include "../../include/agb_canon.h"

namespace agb {

// Programmatic dependent launch: the tick's kernels are launched with the
// programmatic-serialization attribute, so a kernel's CTAs may be scheduled
// while its predecessor on the stream drains. Every such kernel calls
// pdl_wait() before its first memory access; it returns once the predecessor
// grid has completed and its writes are visible (a no-op without the
// attribute). A grid lets its successor launch when its CTAs exit, or earlier
// where it calls pdl_trigger() (after its own wait, so at most one grid runs
// ahead): the successor's CTAs then take free SM slots and wait there. Measured
// per kernel: an early trigger in every tick kernel made the 25k-cell tick
// slower (94.9 against 93.7 us) and the 1M-cell tick no faster, so only the
// FTCS pass on large fields uses it. AGB_NO_PDL=1 launches normally.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

inline bool pdl_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("AGB_NO_PDL");
        on = (e && e[0] == '1') ? 0 : 1;
    }
    return on == 1;
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}


// ---------------------------------------------------------------------------
// Contract SoA (contracts/cell_store_v1.h:42-75), device pointers.
// ---------------------------------------------------------------------------
struct SoA {
    uint64_t* id;
    uint32_t* flags;
    uint8_t* death_cause;
    double *x, *y, *z, *vx, *vy, *vz, *energy;
    float *temp_cell, *emit_power, *dir_x, *dir_y, *dir_z;
    double *biomass, *co2_held;
    float* age_s;
    uint64_t* rng_state;
    float *taxis_memory, *run_timer, *t_local, *irradiance, *co2_local, *n2_local;
};

// Device-resident mutable state. Every per-cell kernel reads the live count
// and the current SoA from here, so population changes (division, compaction)
// never need the host: the whole tick can be replayed as one CUDA graph.
struct DevState {
    SoA cur;            // the live SoA
    SoA spare;          // compaction gathers into this one, then the two swap
    int32_t count;      // live upper bound (CellStore::count)
    int32_t hash_count; // count at the last hash build (ranges to clear next time)
    int32_t births;     // divisions marked this tick
    int32_t deads;      // occupied-but-dead slots this tick
    int32_t dead_slots_prev;
    int32_t divisions_this_window;
    int32_t compact_now;
    int32_t live;
    int64_t deaths_total;
    uint64_t next_id;
    uint64_t tick;
    int32_t n_stamps;   // voxels stamped by the last emission stage
    uint32_t error;     // device error word (first failing check)
    int32_t n_boundary_refine;  // counters of FP64 decision refinements (diagnostics)
    int32_t n_contact_refine;
    int32_t n_shadow_refine;
    uint32_t fin_count;      // CTAs of the division pass that have finished (the last one finalises)
    uint32_t scan_tile;      // next tile of the single-pass scan
    uint32_t scan_done;      // CTAs of the single-pass scan that have finished (the last one resets)
    uint32_t t_deposited;    // 1 when a thermal substep may have left heat in the temperature deposits
    uint32_t t_flush_fin;    // CTAs of the temperature flush that have finished (the last one clears t_deposited)
};

// Immutable per-world constants, passed by value.
struct GridDev {
    float* value;
    float* scratch;
    unsigned long long* deposit;
    int32_t nx, ny, nz, enabled;
    int64_t count;
    float dxf, dzf;      // reference FieldView float dx; dz (3-D)
    float hx, hy, hz;    // half extents as the reference computes them (0.5f * n * dx)
    double dx, dz_eff;
    double scale;
    float inv_scale_f;   // (float)(1 / scale)
    float inv_scale_lo;  // (float)(1 / scale - inv_scale_f): with inv_scale_f, 1 / scale to ~2^-48
    float scale_f;       // (float)scale
    double vol_inv;      // 1 / (dx * dx * dz_eff), rounded once (div_known's reciprocal of the voxel volume)
    double scale_inv;    // 1 / scale, rounded once
};

struct HashDev {
    uint32_t* keys;          // per slot (key_kernel output)
    uint32_t* vals;
    uint32_t* keys_sorted;   // current sorted keys
    uint32_t* vals_sorted;
    uint32_t* keys_prev;     // sorted keys of the previous build (ranges to clear)
    int2* ranges;            // dense bucket table {start, end}
    uint32_t* occ;           // one bit per bucket: occupied in the current build
    float4* rec;             // sorted-order snapshot: offsets from the bucket corner + packed bucket coords
    int32_t fix_k;           // fixed-point exponent K of the corner arithmetic
    float fix_inv_f;         // 2^-K
    double fix_inv;
    long long org_fix[3];    // hash origin, x * 2^K
    long long cell_fix;      // bucket edge, x * 2^K
    float cell_f;            // cell_fix * 2^-K
    int32_t nx, ny, nz, buckets;
    float cellf, inv, ox, oy, oz;
    float margin;            // FP32 bucket-coordinate error bound
};

// Error codes written into DevState::error (first one wins).
enum : uint32_t { ERR_NONE = 0, ERR_BUCKET_RANGE = 1, ERR_CAPACITY = 2, ERR_VOXEL_RANGE = 3 };

__device__ __forceinline__ void set_error(DevState* S, uint32_t code) {
    atomicCAS(&S->error, 0u, code);
}

// ---------------------------------------------------------------------------
// PCG32 per-cell streams (src/core/rng.cuh:23-117), integer-exact.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
struct Pcg {
    uint64_t state, inc;
};
__host__ __device__ __forceinline__ uint32_t pcg_next(Pcg& r) {
    const uint64_t old = r.state;
    r.state = old * 6364136223846793005ull + r.inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
__host__ __device__ __forceinline__ uint64_t cell_stream_inc(uint64_t id) {
    return (splitmix64(id ^ 0xA5A5A5A5DEADBEEFull) << 1u) | 1u;
}
__host__ __device__ __forceinline__ Pcg pcg_seed(uint64_t s, uint64_t q) {
    Pcg r{0ull, (q << 1u) | 1u};
    pcg_next(r);
    r.state += s;
    pcg_next(r);
    return r;
}
__host__ __device__ __forceinline__ uint64_t cell_rng_init(uint64_t seed, uint64_t id) {
    return pcg_seed(seed ^ splitmix64(id), splitmix64(id + 1)).state;
}
__host__ __device__ __forceinline__ uint64_t pcg_split(uint64_t parent, uint64_t did) {
    return splitmix64(parent ^ splitmix64(did * 0x2545F4914F6CDD1Dull));
}
// The 53 random bits of uniform01d (rng.cuh:80-84); the value is bits * 2^-53.
__device__ __forceinline__ uint64_t uniform53(Pcg& r) {
    const uint64_t hi = (uint64_t)pcg_next(r) << 21;
    const uint64_t lo = (uint64_t)pcg_next(r) >> 11;
    return (hi ^ lo) & ((1ull << 53) - 1);
}
__device__ __forceinline__ double uniform01d(Pcg& r) {
    return (double)uniform53(r) * (1.0 / 9007199254740992.0);
}

// Round-to-nearest-even conversions between 64-bit integers and float with
// integer instructions. The hardware's 64-bit integer <-> float conversions
// issue on the FP64 pipe, a small fraction of the FP32 rate on this part;
// these give the same results (round to nearest, ties to even).
__device__ __forceinline__ float u64_to_f(unsigned long long v) {
    if (v < (1ull << 24)) return __uint2float_rn((unsigned int)v);      // exact
    const int lz = __clzll((long long)v);
    const unsigned long long nrm = v << lz;                              // leading one at bit 63
    unsigned int m = (unsigned int)(nrm >> 40);                          // 24 significant bits
    const unsigned long long rest = nrm << 24;                           // the 40 dropped bits
    if (rest > 0x8000000000000000ull || (rest == 0x8000000000000000ull && (m & 1u))) ++m;
    // value m * 2^(e - 23), e = 63 - lz; a carry out of m moves into the exponent
    return __uint_as_float(((unsigned int)(63 - lz + 127) << 23) + m - 0x800000u);
}
__device__ __forceinline__ float ll_to_f(long long v) {
    const float f = u64_to_f(v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v);
    return v < 0 ? -f : f;
}
// float -> int64, round to nearest even (__float2ll_rn) for |v| < 2^63.
__device__ __forceinline__ long long f_to_ll(float v) {
    const unsigned int u = __float_as_uint(v);
    const int ex = (int)((u >> 23) & 0xFFu);
    if (ex >= 127 + 63) return __float2ll_rn(v);                         // out of range, inf, NaN
    if (ex < 126) return 0;                                              // |v| < 0.5
    const unsigned long long m = (u & 0x7FFFFFu) | 0x800000u;            // v = m * 2^(ex - 150)
    const int sh = ex - 150;
    unsigned long long r;
    if (sh >= 0) {
        r = m << sh;
    } else {
        const int rs = -sh;                                              // 1..24
        const unsigned long long q = m >> rs, rem = m & ((1ull << rs) - 1ull), half = 1ull << (rs - 1);
        r = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
    }
    return (u >> 31) ? -(long long)r : (long long)r;
}

// A fixed-point deposit as the flush folds it into a float field:
// (float)((double)raw / scale), from_fixed (fixed_atomic.cuh:31-33) rounded to
// float as flush_kernel does (diffuse.cu:51-60), bit for bit, on the FP32 pipe.
// The quotient is formed as a double-float product of raw (split into two
// floats exactly: hi + remainder) and the scale's reciprocal (inv_hi + inv_lo,
// ~2^-48 relative), to within 2^-44.5 of |raw / scale|, and rounded to float;
// the exact two-sum residual of that rounding shows how far the value lies from
// a rounding midpoint. Only when it lies within the error bound (4 calls in
// 10^6 on random deposits) does the FP64 division decide, out of line. Checked
// on the CPU against the double division on 6.5e7 deposits, random and placed
// next to rounding midpoints, at the three deposit scales: no difference. A plain FP32
// raw * (1 / scale) is off in the last bit often enough that a field drained
// by rationing ended at -4e-9 instead of 0.
static __device__ __noinline__ float fixed_to_f_div(long long raw, double scale) {
    return (float)__ddiv_rn((double)raw, scale);
}
__device__ __forceinline__ float fixed_to_f(long long raw, float inv_hi, float inv_lo, double scale) {
    const float r_hi = ll_to_f(raw);
    const float r_lo = ll_to_f(raw - f_to_ll(r_hi));                     // remainder exact in int64
    const float p = __fmul_rn(r_hi, inv_hi);
    const float e = __fmaf_rn(r_hi, inv_hi, -p);                         // p's rounding error, exact
    const float c = __fadd_rn(e, __fmaf_rn(r_hi, inv_lo, __fmul_rn(r_lo, inv_hi)));
    const float f = __fadd_rn(p, c);
    const float bb = __fsub_rn(f, p);
    const float t = __fadd_rn(__fsub_rn(p, __fsub_rn(f, bb)), __fsub_rn(c, bb));   // (p + c) - f, exact
    // The midpoints next to f lie half an ulp away (a quarter below an exact
    // power of two, whose lower neighbour is closer); f stands when |t| plus
    // the bound on the product's error and on the reference's own rounding to
    // double stays short of that.
    const float af = fabsf(f);
    const uint32_t ab = __float_as_uint(af);
    const float lim = __uint_as_float(ab & 0x7F800000u) * ((ab & 0x7FFFFFu) ? 0x1p-24f : 0x1p-25f);
    if (fabsf(t) + af * 0x1p-43f < lim) return f;
    return fixed_to_f_div(raw, scale);
}

// FP64 draws as the reference takes them (rng.cuh:86-101), for the seeded
// spawns and the predators: explicitly rounded, CUDA's log/cos/sin.
__device__ __forceinline__ double uniform_range(Pcg& r, double lo, double hi) {   // rng.cuh:86-88
    return __dadd_rn(lo, __dmul_rn(__dsub_rn(hi, lo), uniform01d(r)));
}
__device__ __forceinline__ void gaussian_pair_d(Pcg& r, double& z0, double& z1) {
    double u1 = uniform01d(r);
    if (u1 < 1.0e-300) u1 = 1.0e-300;
    const double u2 = uniform01d(r);
    const double mag = sqrt(__dmul_rn(-2.0, log(u1)));
    const double ang = __dmul_rn(6.283185307179586476925286766559, u2);
    z0 = __dmul_rn(mag, cos(ang));
    z1 = __dmul_rn(mag, sin(ang));
}

// Box-Muller in FP32 from the reference's 53-bit uniforms (rng.cuh:92-101).
// ln(u1) is taken as log1p(-(1-u1)) for u1 > 1/2, with 1-u1 exact in integers,
// so the magnitude keeps ~1e-7 relative accuracy near u1 = 1. The reference
// floors u1 at 1e-300; here the floor is the smallest 53-bit uniform (2^-53),
// which differs only for u1 == 0 (probability 2^-53).
__device__ __forceinline__ void gaussian_pair_f(Pcg& r, float& z0, float& z1) {
    uint64_t b1 = uniform53(r);
    const uint64_t b2 = uniform53(r);
    float lg;
    if (b1 == 0ull) b1 = 1ull;
    if (b1 > (1ull << 52)) {
        const float w = u64_to_f((1ull << 53) - b1) * 1.1102230246251565e-16f;  // 1 - u1, exact bits
        lg = log1pf(-w);
    } else {
        lg = logf(u64_to_f(b1) * 1.1102230246251565e-16f);
    }
    const float mag = sqrtf(-2.0f * lg);
    float s, c;
    sincospif(u64_to_f(b2) * 2.220446049250313e-16f, &s, &c);   // angle = 2*pi*u2
    z0 = mag * c;
    z1 = mag * s;
}

// ---------------------------------------------------------------------------
// Fixed point (src/core/fixed_atomic.cuh:27-45).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void deposit_fixed(unsigned long long* acc, long long v) {
    atomicAdd(acc, (unsigned long long)v);
}
// FP32 value -> fixed point (llround semantics except exact .5 ties).
__device__ __forceinline__ long long to_fixed_f(float v, float scale) {
    return f_to_ll(v * scale);
}

// ---------------------------------------------------------------------------
// Exactly-rounded FP32 helpers: the reference's float expressions evaluated in
// C order with no contraction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// grid_sample bilinear body (src/fields/grid.cuh:109-125).
__device__ __forceinline__ float bilerp(const float* __restrict__ v, int32_t nx, int32_t ny, int32_t x0,
                                        int32_t y0, float tx, float ty) {
    const int32_t x1 = x0 + 1, y1 = y0 + 1;
    const int32_t xa = x0 < 0 ? 0 : (x0 >= nx ? nx - 1 : x0), xb = x1 < 0 ? 0 : (x1 >= nx ? nx - 1 : x1);
    const int32_t ya = y0 < 0 ? 0 : (y0 >= ny ? ny - 1 : y0), yb = y1 < 0 ? 0 : (y1 >= ny ? ny - 1 : y1);
    const float v00 = __ldg(v + (int64_t)ya * nx + xa), v10 = __ldg(v + (int64_t)ya * nx + xb);
    const float v01 = __ldg(v + (int64_t)yb * nx + xa), v11 = __ldg(v + (int64_t)yb * nx + xb);
    const float omx = fs(1.0f, tx), omy = fs(1.0f, ty);
    float r = fm(fm(omx, omy), v00);
    r = fa(r, fm(fm(tx, omy), v10));
    r = fa(r, fm(fm(omx, ty), v01));
    r = fa(r, fm(fm(tx, ty), v11));
    return r;
}

// grid_sample; for nz > 1 a z-lerp of two bilinears (the 3-D extension).
__device__ __forceinline__ float grid_sample(const GridDev& g, const float* __restrict__ val, float x,
                                             float y, float z) {
    const float gx = fs(fd(fa(x, g.hx), g.dxf), 0.5f);
    const float gy = fs(fd(fa(y, g.hy), g.dxf), 0.5f);
    const int32_t x0 = (int32_t)floorf(gx), y0 = (int32_t)floorf(gy);
    const float tx = fs(gx, (float)x0), ty = fs(gy, (float)y0);
    if (g.nz == 1) return bilerp(val, g.nx, g.ny, x0, y0, tx, ty);
    const float gz = fs(fd(fa(z, g.hz), g.dzf), 0.5f);
    const int32_t z0 = (int32_t)floorf(gz);
    const float tz = fs(gz, (float)z0);
    const int32_t za = z0 < 0 ? 0 : (z0 >= g.nz ? g.nz - 1 : z0);
    const int32_t zb = z0 + 1 < 0 ? 0 : (z0 + 1 >= g.nz ? g.nz - 1 : z0 + 1);
    const int64_t plane = (int64_t)g.nx * g.ny;
    const float b0 = bilerp(val + za * plane, g.nx, g.ny, x0, y0, tx, ty);
    const float b1 = bilerp(val + zb * plane, g.nx, g.ny, x0, y0, tx, ty);
    return fa(fm(fs(1.0f, tz), b0), fm(tz, b1));
}

// grid_index_nearest (src/fields/grid.cuh:134-141); k from z for nz > 1.
__device__ __forceinline__ int64_t grid_nearest(const GridDev& g, float x, float y, float z) {
    int32_t i = (int32_t)fd(fa(x, g.hx), g.dxf);
    int32_t j = (int32_t)fd(fa(y, g.hy), g.dxf);
    i = i < 0 ? 0 : (i >= g.nx ? g.nx - 1 : i);
    j = j < 0 ? 0 : (j >= g.ny ? g.ny - 1 : j);
    int32_t k = 0;
    if (g.nz > 1) {
        k = (int32_t)fd(fa(z, g.hz), g.dzf);
        k = k < 0 ? 0 : (k >= g.nz ? g.nz - 1 : k);
    }
    return (int64_t)i + (int64_t)g.nx * ((int64_t)j + (int64_t)g.ny * k);
}

// ---------------------------------------------------------------------------
// Double -> float pair without FP64 instructions: hi holds the top 24 bits of
// the significand (truncated, exact), lo the next bits rounded to 24. hi + lo
// reproduces x to ~2^-48 relative; differences of nearby positions computed as
// (hi_i - hi_j) + (lo_i - lo_j) are then accurate to ~1e-12 of a cell diameter.
// |x| below 2^-100 maps to 0 (positions are never that small and nonzero).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void split_double(double x, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    if (e < -100) { hi = 0.0f; lo = 0.0f; return; }
    const unsigned int sign = (unsigned int)(b >> 63) << 31;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    hi = __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | (unsigned int)(m >> 29));
    const unsigned int low = (unsigned int)(m & 0x1FFFFFFFull);
    // low * 2^(e - 52), built as a power-of-two float factor (e - 52 >= -152;
    // e >= -100 keeps the factor normal: -152 + ... handled by two steps).
    const float p1 = __uint_as_float((unsigned int)(e - 52 + 127 + 60) << 23);  // 2^(e-52+60)
    const float f = (float)low * p1 * 8.673617379884035e-19f;                     // * 2^-60
    lo = sign ? -f : f;
}

// Round-to-nearest double -> float with integer instructions (same result as
// static_cast<float>(double) for values in the float normal range; the rare
// others go through the hardware conversion).
__device__ __forceinline__ float d2f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    if (e < -126 || e > 127) return __double2float_rn(x);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    unsigned int f = ((unsigned int)(b >> 63) << 31) | ((unsigned int)(e + 127) << 23) | (unsigned int)(m >> 29);
    const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFull);
    if (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) f += 1u;
    return __uint_as_float(f);
}

// Exact float -> double with integer instructions (normal floats; others via hardware).
__device__ __forceinline__ double f2d(float v) {
    const unsigned int u = __float_as_uint(v);
    const unsigned int ex = (u >> 23) & 0xFFu;
    if (ex == 0u || ex == 0xFFu) return (double)v;
    const unsigned long long b = ((unsigned long long)(u >> 31) << 63) |
                                 ((unsigned long long)(ex - 127u + 1023u) << 52) |
                                 ((unsigned long long)(u & 0x7FFFFFu) << 29);
    return __longlong_as_double((long long)b);
}

// ---------------------------------------------------------------------------
// Spatial hash coordinate (src/sim/hash.cuh:63-68): (int)((x - o) * inv) in
// FP64, clamped. The FP32 estimate decides unless it lies within `margin` of
// an integer boundary, where the FP64 expression settles it.
// ---------------------------------------------------------------------------
// The FP64 expression, out of line so that it runs only in warps where a lane
// needs it (inline, the compiler may evaluate it for every lane, and FP64
// issues at a small fraction of the FP32 rate).
static __device__ __noinline__ int32_t hash_axis_fp64(double x, float o, float inv) {
    return (int32_t)((x - (double)o) * (double)inv);
}

__device__ __forceinline__ int32_t hash_axis(double x, float o, float inv, int32_t n, float margin) {
    float hi, lo;
    split_double(x, hi, lo);
    const float v = (hi - o + lo) * inv;
    const float fl = floorf(v);
    int32_t c;
    if (v - fl > margin && (fl + 1.0f) - v > margin && fabsf(v) > margin) {
        c = (int32_t)fl;                     // v > 0 here or clamps to 0 below
        if (v < 0.0f) c = -1;
    } else {
        c = hash_axis_fp64(x, o, inv);
    }
    return c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
}

__device__ __forceinline__ void hash_coords(const HashDev& h, double x, double y, double z, int32_t& gx,
                                            int32_t& gy, int32_t& gz) {
    gx = hash_axis(x, h.ox, h.inv, h.nx, h.margin);
    gy = hash_axis(y, h.oy, h.inv, h.ny, h.margin);
    gz = hash_axis(z, h.oz, h.inv, h.nz, h.margin);
}

// Position as 64-bit fixed point X = x * 2^K (integer instructions only), with
// K chosen per world so the chamber's half extent fits 63 bits (K = 70 for a
// 4 mm chamber). Exact for |x| >= 2^(52-K) (3.8 um at K = 70); below that the
// dropped bits are worth less than 2^-K m. Differences of two such values are
// exact integers, so neighbour separations carry no cancellation error, and
// (double)(Xi - Xj) * 2^-K is the correctly rounded x_i - x_j the reference
// forms in FP64.
__device__ __forceinline__ long long to_fix64(double x, int K) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ef = (int)((b >> 52) & 0x7FF);
    if (ef == 0) return 0;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int sh = ef - 1023 - 52 + K;
    long long X;
    if (sh >= 0) X = (long long)(m << (sh > 10 ? 10 : sh));   // |x| within the chamber keeps sh <= 10
    else if (sh > -64) X = (long long)(m >> (-sh));
    else X = 0;
    return (b >> 63) ? -X : X;
}
__device__ __forceinline__ float fix_diff_f(long long d, float inv) { return ll_to_f(d) * inv; }
__device__ __forceinline__ double fix_diff_d(long long d, double inv) { return __dmul_rn((double)d, inv); }

// column_transmittance of a stamped voxel (src/sim/emission.cuh:43-47) from
// its fixed-point stamp: 1 - area / face, floored at 0. The same FP64
// operations on the host and the device.
__host__ __device__ inline double occlusion_of(long long dep, double scale, double face) {
    const double area = (double)dep / scale;
    const double tr = 1.0 - area / face;
    return tr > 0.0 ? tr : 0.0;
}

// a / b rounded to nearest for a divisor known ahead, y = 1 / b rounded to
// nearest (computed on the host): Markstein's correction step (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990): q = a y, r = a - b q by FMA,
// q1 = q + r y by FMA. q1 is returned only where an exact test shows it is
// the nearest double to a / b: q1 normal and not a power of two (its
// neighbours an ulp away on both sides), h = b ulp(q1) / 2 formed exactly (b
// times a power of two, a normal result), and |RN(a - b q1)| < h, which by the
// monotonicity of rounding implies |a / b - q1| < ulp(q1) / 2. Anything else
// (ties, binade edges, zero, extreme exponents, a stale y) takes the IEEE
// division, so the result is the correctly rounded quotient in every case.
static __device__ __noinline__ double div_known_ieee(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double div_known(double a, double b, double y) {
    const double q = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-b, q, a), y, q);
    const unsigned long long bits = (unsigned long long)__double_as_longlong(q1);
    const int e = (int)((bits >> 52) & 0x7FFu);
    if (e > 53 && e < 2047 && (bits & 0xFFFFFFFFFFFFFull) != 0ull) {
        const double h = __dmul_rn(b, __longlong_as_double((long long)(e - 53) << 52));
        if (h >= 2.2250738585072014e-308 && fabs(__fma_rn(-b, q1, a)) < h) return q1;
    }
    return div_known_ieee(a, b);
}

// Order-preserving map of a double onto uint64: compares of finite doubles
// become integer compares (no FP64 pipe).
__device__ __forceinline__ unsigned long long dkey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Grid-stride helpers.
#define AGB_FOR_CELLS(i, n) \
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// The block a kernel body works as: a plain launch over one world uses its
// own grid; a batched launch over many chambers gives each chamber a run of
// the grid's blocks, and a body sees only its chamber's block index and count.
struct Blk {
    int32_t x, n;
};
__device__ __forceinline__ Blk grid_blk() { return Blk{(int32_t)blockIdx.x, (int32_t)gridDim.x}; }
#define AGB_FOR_CELLS_B(i_, blk_, count_)                                                      \
    for (int32_t i_ = (blk_).x * (int32_t)blockDim.x + (int32_t)threadIdx.x; i_ < (count_); \
         i_ += (blk_).n * (int32_t)blockDim.x)

// Block map of a batched launch: entry k = (chamber << 16) | (block within the
// chamber) for block k of the grid.
__device__ __forceinline__ void batch_block(const uint32_t* __restrict__ map, int32_t& ch, int32_t& x) {
    const uint32_t m = __ldg(&map[blockIdx.x]);
    ch = (int32_t)(m >> 16);
    x = (int32_t)(m & 0xFFFFu);
}

}  // namespace agb
