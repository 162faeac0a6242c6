/*
 * oracle/oracle.c -- CPU oracle of the per-tick physics step (test infrastructure).
 *
 * A plain-C restatement of the reference's kernel bodies in the reference's own
 * FP64 arithmetic; each function names the reference file:line it follows.
 * Float expressions are written in the reference's evaluation order and the
 * file is compiled with -ffp-contract=off, so FP32 field arithmetic matches the
 * reference (and the CUDA engine, which uses explicitly rounded operations)
 * bit for bit. Generalisations beyond the reference (3-D grids, per-face
 * boundary conditions, a z light axis, the energy division predicate, the
 * compaction period, the extra spawn distributions) are marked EXTENSION.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/agb_canon.h"

/* ------------------------------------------------------------------------- */
/* RNG: src/core/rng.cuh:23-117                                               */
/* ------------------------------------------------------------------------- */
typedef struct { uint64_t state, inc; } pcg32;

static uint64_t splitmix64(uint64_t x) {                  /* rng.cuh:23-28 */
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static uint32_t pcg32_next(pcg32* r) {                    /* rng.cuh:35-41 */
    const uint64_t old = r->state;
    r->state = old * 6364136223846793005ull + r->inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

static pcg32 pcg32_seed(uint64_t initstate, uint64_t initseq) {   /* rng.cuh:44-50 */
    pcg32 r = {0ull, (initseq << 1u) | 1u};
    pcg32_next(&r);
    r.state += initstate;
    pcg32_next(&r);
    return r;
}

static uint64_t cell_stream_inc(uint64_t id) {            /* rng.cuh:54-56 */
    return (splitmix64(id ^ 0xA5A5A5A5DEADBEEFull) << 1u) | 1u;
}
static pcg32 cell_rng(uint64_t state, uint64_t id) {      /* rng.cuh:58-60 */
    pcg32 r = {state, cell_stream_inc(id)};
    return r;
}
static uint64_t cell_rng_init(uint64_t seed, uint64_t id) {   /* rng.cuh:62-65 */
    return pcg32_seed(seed ^ splitmix64(id), splitmix64(id + 1)).state;
}
static uint64_t pcg_split(uint64_t parent, uint64_t did) {    /* rng.cuh:69-71 */
    return splitmix64(parent ^ splitmix64(did * 0x2545F4914F6CDD1Dull));
}
static double uniform01d(pcg32* r) {                      /* rng.cuh:80-84 */
    const uint64_t hi = (uint64_t)pcg32_next(r) << 21;
    const uint64_t lo = (uint64_t)pcg32_next(r) >> 11;
    return (double)((hi ^ lo) & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}
static double uniform_range(pcg32* r, double lo, double hi) {   /* rng.cuh:86-88 */
    return lo + (hi - lo) * uniform01d(r);
}
static void gaussian_pair(pcg32* r, double* z0, double* z1) {   /* rng.cuh:92-101 */
    double u1 = uniform01d(r);
    if (u1 < 1.0e-300) u1 = 1.0e-300;
    const double u2 = uniform01d(r);
    const double mag = sqrt(-2.0 * log(u1));
    const double ang = 6.283185307179586476925286766559 * u2;
    *z0 = mag * cos(ang);
    *z1 = mag * sin(ang);
}
static double gaussian(pcg32* r) { double a, b; gaussian_pair(r, &a, &b); return a; }

void orc_pcg32_seed_draws(uint64_t s, uint64_t q, int32_t n, uint32_t* out) {
    pcg32 r = pcg32_seed(s, q);
    for (int32_t i = 0; i < n; ++i) out[i] = pcg32_next(&r);
}
uint64_t orc_cell_rng_init(uint64_t seed, uint64_t id) { return cell_rng_init(seed, id); }
uint64_t orc_pcg_split(uint64_t p, uint64_t d) { return pcg_split(p, d); }

/* ------------------------------------------------------------------------- */
/* Small vector + fixed point: src/core/vec.cuh, src/core/fixed_atomic.cuh    */
/* ------------------------------------------------------------------------- */
typedef struct { double x, y, z; } vec3;
static vec3 v3(double x, double y, double z) { vec3 r = {x, y, z}; return r; }
static vec3 vsub(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static vec3 vscale(vec3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static double vdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static vec3 vnormalize(vec3 a) {                          /* vec.cuh:34-37 */
    const double l = sqrt(vdot(a, a));
    return l > 0.0 ? vscale(a, 1.0 / l) : v3(0.0, 0.0, 1.0);
}

static int64_t to_fixed(double v, double scale) { return (int64_t)llround(v * scale); } /* fixed_atomic.cuh:27-29 */
static double from_fixed(uint64_t raw, double scale) { return (double)(int64_t)raw / scale; } /* :31-33 */

static void deposit_add(uint64_t* acc, double value, double scale) {   /* fixed_atomic.cuh:38-40 */
    const uint64_t v = (uint64_t)to_fixed(value, scale);
#ifdef _OPENMP
#pragma omp atomic
#endif
    *acc += v;
}

/* ------------------------------------------------------------------------- */
/* Grids: src/fields/grid.cuh, src/fields/diffuse.cu                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    int enabled;
    int32_t nx, ny, nz;
    int64_t count;
    double dx, dz, dz_eff, diffusivity, deposit_scale, robin;
    float dxf, dzf, robinf;
    int32_t bc[6];
    float facef[6];
    float* value;
    float* scratch;
    uint64_t* deposit;
} grid;

static int grid_init(grid* g, const agb_grid_desc* d, double chamber_w, double chamber_d) {
    memset(g, 0, sizeof(*g));
    if (d->nx <= 0) return 0;
    if (d->nx <= 1 || d->ny <= 1 || d->nz < 1) return AGB_INVALID_ARGUMENT;   /* diffuse.cu:94 */
    g->enabled = 1;
    g->nx = d->nx; g->ny = d->ny; g->nz = d->nz;
    g->count = (int64_t)d->nx * d->ny * d->nz;
    g->dx = chamber_w / (double)d->nx;                     /* diffuse.cu:97 */
    g->dz_eff = chamber_d / (double)d->nz;                 /* nz == 1: the full depth */
    g->dz = d->nz > 1 ? g->dz_eff : 0.0;
    if (d->nz > 1 && fabs(g->dz / g->dx - 1.0) > 1e-9) return AGB_UNSUPPORTED;
    g->diffusivity = d->diffusivity;
    g->deposit_scale = d->deposit_scale;
    g->robin = g->dx * AGB_AIR_CONVECTION_H / AGB_WATER_CONDUCTIVITY;   /* diffuse.cu:102 */
    g->dxf = (float)g->dx;                                  /* grid_view, diffuse.cu:198 */
    g->dzf = (float)g->dz;
    g->robinf = (float)g->robin;
    for (int f = 0; f < 6; ++f) { g->bc[f] = d->bc[f]; g->facef[f] = (float)d->face_value[f]; }
    g->value = (float*)malloc(sizeof(float) * g->count);
    g->scratch = (float*)malloc(sizeof(float) * g->count);
    g->deposit = (uint64_t*)calloc((size_t)g->count, sizeof(uint64_t));
    if (!g->value || !g->scratch || !g->deposit) return AGB_OUT_OF_MEMORY;
    const float fill = (float)d->init;                      /* grid_fill, diffuse.cu:128-134 */
    for (int64_t i = 0; i < g->count; ++i) g->value[i] = g->scratch[i] = fill;
    return 0;
}

static void grid_free(grid* g) { free(g->value); free(g->scratch); free(g->deposit); }

/* grid_sample, grid.cuh:109-125 (bilinear); EXTENSION: trilinear for nz > 1
 * as a z-lerp of two reference bilinears. */
static float bilerp(const float* v, int32_t nx, int32_t ny, int32_t x0, int32_t y0, float tx, float ty) {
    const int32_t x1 = x0 + 1, y1 = y0 + 1;
    const int32_t xa = x0 < 0 ? 0 : (x0 >= nx ? nx - 1 : x0), xb = x1 < 0 ? 0 : (x1 >= nx ? nx - 1 : x1);
    const int32_t ya = y0 < 0 ? 0 : (y0 >= ny ? ny - 1 : y0), yb = y1 < 0 ? 0 : (y1 >= ny ? ny - 1 : y1);
    return (1.0f - tx) * (1.0f - ty) * v[ya * nx + xa] + tx * (1.0f - ty) * v[ya * nx + xb] +
           (1.0f - tx) * ty * v[yb * nx + xa] + tx * ty * v[yb * nx + xb];
}

static float grid_sample(const grid* g, float x, float y, float z) {
    const float hx = 0.5f * g->nx * g->dxf;
    const float hy = 0.5f * g->ny * g->dxf;
    const float gx = (x + hx) / g->dxf - 0.5f;
    const float gy = (y + hy) / g->dxf - 0.5f;
    const int32_t x0 = (int32_t)floorf(gx);
    const int32_t y0 = (int32_t)floorf(gy);
    const float tx = gx - (float)x0;
    const float ty = gy - (float)y0;
    if (g->nz == 1) return bilerp(g->value, g->nx, g->ny, x0, y0, tx, ty);
    const float hz = 0.5f * g->nz * g->dzf;
    const float gz = (z + hz) / g->dzf - 0.5f;
    const int32_t z0 = (int32_t)floorf(gz);
    const float tz = gz - (float)z0;
    const int32_t za = z0 < 0 ? 0 : (z0 >= g->nz ? g->nz - 1 : z0);
    const int32_t zb = z0 + 1 < 0 ? 0 : (z0 + 1 >= g->nz ? g->nz - 1 : z0 + 1);
    const int64_t plane = (int64_t)g->nx * g->ny;
    const float b0 = bilerp(g->value + za * plane, g->nx, g->ny, x0, y0, tx, ty);
    const float b1 = bilerp(g->value + zb * plane, g->nx, g->ny, x0, y0, tx, ty);
    return (1.0f - tz) * b0 + tz * b1;
}

/* grid_index_nearest, grid.cuh:134-141; EXTENSION: k from z for nz > 1. */
static int64_t grid_nearest(const grid* g, float x, float y, float z) {
    const float hx = 0.5f * g->nx * g->dxf;
    const float hy = 0.5f * g->ny * g->dxf;
    int32_t i = (int32_t)((x + hx) / g->dxf);
    int32_t j = (int32_t)((y + hy) / g->dxf);
    i = i < 0 ? 0 : (i >= g->nx ? g->nx - 1 : i);
    j = j < 0 ? 0 : (j >= g->ny ? g->ny - 1 : j);
    int32_t k = 0;
    if (g->nz > 1) {
        const float hz = 0.5f * g->nz * g->dzf;
        k = (int32_t)((z + hz) / g->dzf);
        k = k < 0 ? 0 : (k >= g->nz ? g->nz - 1 : k);
    }
    return (int64_t)i + (int64_t)g->nx * ((int64_t)j + (int64_t)g->ny * k);
}

/* flush_kernel, diffuse.cu:51-60 */
static void grid_flush(grid* g) {
    if (!g->enabled) return;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < g->count; ++i) {
        const uint64_t raw = g->deposit[i];
        if (raw != 0ull) {
            g->value[i] += (float)from_fixed(raw, g->deposit_scale);
            g->deposit[i] = 0ull;
        }
    }
}

/* diffuse_kernel's ghost, diffuse.cu:27-36, per face (EXTENSION: a bc per face). */
static float ghost(const grid* g, int face, float c) {
    if (g->bc[face] == AGB_BC_DIRICHLET) return g->facef[face];
    if (g->bc[face] == AGB_BC_ROBIN) return c - g->robinf * (c - g->facef[face]);
    return c;
}

/* diffuse_kernel, diffuse.cu:19-44: one explicit pass value -> scratch, then the
 * ping-pong swap of grid_diffuse_substep (:153-155). EXTENSION: 7-point for nz > 1. */
static void grid_pass(grid* g, float coeff) {
    const int32_t nx = g->nx, ny = g->ny, nz = g->nz;
    const int64_t plane = (int64_t)nx * ny;
    const float* src = g->value;
    float* dst = g->scratch;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) collapse(2)
#endif
    for (int32_t k = 0; k < nz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) {
                const int64_t idx = (int64_t)i + (int64_t)nx * j + plane * k;
                const float c = src[idx];
                const float l = (i > 0) ? src[idx - 1] : ghost(g, AGB_FACE_XMIN, c);
                const float r = (i < nx - 1) ? src[idx + 1] : ghost(g, AGB_FACE_XMAX, c);
                const float d = (j > 0) ? src[idx - nx] : ghost(g, AGB_FACE_YMIN, c);
                const float u = (j < ny - 1) ? src[idx + nx] : ghost(g, AGB_FACE_YMAX, c);
                if (nz == 1) {
                    dst[idx] = c + coeff * (l + r + d + u - 4.0f * c);
                } else {
                    const float b = (k > 0) ? src[idx - plane] : ghost(g, AGB_FACE_ZMIN, c);
                    const float f = (k < nz - 1) ? src[idx + plane] : ghost(g, AGB_FACE_ZMAX, c);
                    dst[idx] = c + coeff * (l + r + d + u + b + f - 6.0f * c);
                }
            }
    float* t = g->value; g->value = g->scratch; g->scratch = t;
}

/* substeps_for_dt, grid.cuh:51-53; 3-D uses the 1/6 bound (EXTENSION). */
static int32_t grid_substeps(const grid* g, double dt) {
    const double lim = g->nz > 1 ? 6.0 : 4.0;
    return (int32_t)(dt / (g->dx * g->dx / (lim * g->diffusivity))) + 1;
}
static float grid_coeff(const grid* g, double dt_sub) {
    return (float)(g->diffusivity * dt_sub / (g->dx * g->dx));     /* diffuse.cu:145,167 */
}
static int coeff_stable(const grid* g, float c) {
    return g->nz > 1 ? (c <= (float)(1.0 / 6.0)) : (c <= 0.25f);   /* diffuse.cu:146,172 */
}

/* grid_diffuse, diffuse.cu:159-186 */
static int grid_diffuse(grid* g, double dt) {
    if (!g->enabled) return 0;
    const int32_t steps = grid_substeps(g, dt);
    if (steps <= 0) return 0;
    const double dt_sub = dt / steps;
    const float coeff = grid_coeff(g, dt_sub);
    if (!coeff_stable(g, coeff)) return AGB_INVALID_ARGUMENT;
    for (int32_t s = 0; s < steps; ++s) grid_pass(g, coeff);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* World                                                                      */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t* id; uint32_t* flags; uint8_t* death_cause;
    double *x, *y, *z, *vx, *vy, *vz, *energy;
    float *temp_cell, *emit_power, *dir_x, *dir_y, *dir_z;
    double *biomass, *co2_held;
    float* age_s;
    uint64_t* rng_state;
    float *taxis_memory, *run_timer, *t_local, *irradiance, *co2_local, *n2_local;
} soa;

/* TaumoebaStore (src/sim/predation.cuh:85-105): the predator's 20 arrays. */
typedef struct {
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
} tau_soa;
static const size_t TAU_SZ[20] = {8, 4, 8, 8, 8, 8, 8, 8, 4, 4, 4, 8, 8, 4, 4, 4, 8, 4, 4, 4};
static void tau_ptrs(tau_soa* t, void** p[20]) {
    void** q[20] = {(void**)&t->id, (void**)&t->flags, (void**)&t->x, (void**)&t->y, (void**)&t->z,
                    (void**)&t->vx, (void**)&t->vy, (void**)&t->vz, (void**)&t->dir_x, (void**)&t->dir_y,
                    (void**)&t->dir_z, (void**)&t->biomass, (void**)&t->prey_biomass, (void**)&t->digest_timer,
                    (void**)&t->tolerance, (void**)&t->generation, (void**)&t->rng_state,
                    (void**)&t->density_ema, (void**)&t->run_timer, (void**)&t->target};
    memcpy(p, q, sizeof(q));
}

struct orc_world {
    agb_world_desc d;
    soa c;
    int32_t count, capacity;
    uint64_t next_id;
    grid g[AGB_FIELD_COUNT];
    /* hash (src/sim/hash.cuh:25-48) */
    int32_t hnx, hny, hnz, hbuckets;
    double hcell;
    float hcellf, hinv, hox, hoy, hoz;
    uint32_t *keys, *vals, *keys_sorted, *vals_sorted, *tmp_k, *tmp_v;
    int32_t *bstart, *bend;
    double *fx, *fy, *fz;
    /* Checker-only: per cell, the summed magnitudes of the terms behind the
     * last motion stage's force, velocity and displacement (see motion_step). */
    double *fscale, *vscale, *pscale;
    uint64_t* co2_demand;
    int32_t *scan_flags, *prefix, *compact_src;
    void* scratch;
    /* counters (World, src/sim/world.cuh:111-129) */
    int32_t divisions_this_window, dead_slots_prev;
    int64_t deaths_total, deaths_reported;
    uint64_t tick;
    double sim_time, physics_rate, biology_rate;
    uint64_t accum[12];
    /* the spin-drive flash (World::flash_active, petrova_flash_power, d_flash_accum) */
    int flash_active;
    double flash_power;
    uint64_t flash_accum[4];
    /* the predator store, its next id and the per-cell claim words */
    tau_soa t;
    int32_t tau_count, tau_capacity;
    uint64_t tau_next_id;
    uint64_t* claim;
};

static void soa_sizes(size_t sz[25]) {
    const size_t s[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};
    memcpy(sz, s, sizeof(s));
}
static void soa_ptrs(soa* c, void** p) {
    void** q[25] = {(void**)&c->id, (void**)&c->flags, (void**)&c->death_cause, (void**)&c->x,
                    (void**)&c->y, (void**)&c->z, (void**)&c->vx, (void**)&c->vy, (void**)&c->vz,
                    (void**)&c->energy, (void**)&c->temp_cell, (void**)&c->emit_power,
                    (void**)&c->dir_x, (void**)&c->dir_y, (void**)&c->dir_z, (void**)&c->biomass,
                    (void**)&c->co2_held, (void**)&c->age_s, (void**)&c->rng_state,
                    (void**)&c->taxis_memory, (void**)&c->run_timer, (void**)&c->t_local,
                    (void**)&c->irradiance, (void**)&c->co2_local, (void**)&c->n2_local};
    for (int k = 0; k < 25; ++k) p[k] = (void*)q[k];
}
static void host_ptrs(const agb_cells* h, void** p) {
    void* q[25] = {h->id, h->flags, h->death_cause, h->x, h->y, h->z, h->vx, h->vy, h->vz,
                   h->energy, h->temp_cell, h->emit_power, h->dir_x, h->dir_y, h->dir_z,
                   h->biomass, h->co2_held, h->age_s, h->rng_state, h->taxis_memory,
                   h->run_timer, h->t_local, h->irradiance, h->co2_local, h->n2_local};
    memcpy(p, q, sizeof(q));
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

void orc_world_destroy(orc_world* w) {
    if (!w) return;
    void* p[25];
    soa_ptrs(&w->c, p);
    for (int k = 0; k < 25; ++k) free(*(void**)p[k]);
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) grid_free(&w->g[f]);
    free(w->keys); free(w->vals); free(w->keys_sorted); free(w->vals_sorted);
    free(w->tmp_k); free(w->tmp_v); free(w->bstart); free(w->bend);
    free(w->fx); free(w->fy); free(w->fz); free(w->co2_demand);
    free(w->fscale); free(w->vscale); free(w->pscale);
    free(w->scan_flags); free(w->prefix); free(w->compact_src); free(w->scratch);
    void** tp[20];
    tau_ptrs(&w->t, tp);
    for (int k = 0; k < 20; ++k) free(*tp[k]);
    free(w->claim);
    free(w);
}

/* world_create (src/sim/step.cu:9-78) + hash_create (src/sim/hash.cu:46-80). */
int orc_world_create(const agb_world_desc* d, orc_world** out) {
    *out = NULL;
    if (!d || d->abi_version != AGB_ABI_VERSION) return AGB_CONTRACT_VERSION_MISMATCH;
    if (d->capacity <= 0 || d->capacity > AGB_MAX_CELLS) return AGB_INVALID_ARGUMENT;  /* cell_store.cu:140-141 */
    orc_world* w = (orc_world*)calloc(1, sizeof(orc_world));
    if (!w) return AGB_OUT_OF_MEMORY;
    w->d = *d;
    w->capacity = d->capacity;
    w->next_id = 1;                                      /* cell_store.cuh:42 */
    w->flash_power = AGB_PETROVA_FLASH_POWER;            /* World::petrova_flash_power */
    size_t sz[25];
    soa_sizes(sz);
    void* p[25];
    soa_ptrs(&w->c, p);
    for (int k = 0; k < 25; ++k) {
        *(void**)p[k] = calloc((size_t)d->capacity, sz[k]);
        if (!*(void**)p[k]) { orc_world_destroy(w); return AGB_OUT_OF_MEMORY; }
    }
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) {
        const int rc = grid_init(&w->g[f], &d->grid[f], d->chamber_w, d->chamber_d);
        if (rc) { orc_world_destroy(w); return rc; }
    }
    /* taumoeba_create (predation.cu:306-418) */
    w->tau_capacity = d->tau_capacity > 0 ? d->tau_capacity : AGB_DEFAULT_TAUMOEBA;
    if (w->tau_capacity > AGB_MAX_TAUMOEBA) { orc_world_destroy(w); return AGB_INVALID_ARGUMENT; }
    w->tau_next_id = 1;
    {
        void** tp[20];
        tau_ptrs(&w->t, tp);
        for (int k = 0; k < 20; ++k) {
            *tp[k] = calloc((size_t)w->tau_capacity, TAU_SZ[k]);
            if (!*tp[k]) { orc_world_destroy(w); return AGB_OUT_OF_MEMORY; }
        }
        w->claim = (uint64_t*)calloc((size_t)d->capacity, 8);
        if (!w->claim) { orc_world_destroy(w); return AGB_OUT_OF_MEMORY; }
    }
    const double cell = d->hash_cell_size > 0.0 ? d->hash_cell_size
                                                : AGB_HASH_CELL_FACTOR * AGB_CELL_DIAMETER;
    w->hcell = cell;
    w->hnx = (int32_t)ceil(d->chamber_w / cell);          /* hash.cu:48-53 */
    w->hny = (int32_t)ceil(d->chamber_h / cell);
    w->hnz = (int32_t)ceil(d->chamber_d / cell);
    if (w->hnx < 1) w->hnx = 1;
    if (w->hny < 1) w->hny = 1;
    if (w->hnz < 1) w->hnz = 1;
    const double nb = (double)w->hnx * w->hny * w->hnz;
    if (nb >= 2147483647.0) { orc_world_destroy(w); return AGB_INVALID_ARGUMENT; }
    w->hbuckets = w->hnx * w->hny * w->hnz;
    w->hcellf = (float)cell;                              /* hash_view, hash.cu:90-104 */
    w->hinv = (float)(1.0 / cell);
    w->hox = (float)(-0.5 * w->hnx * cell);
    w->hoy = (float)(-0.5 * w->hny * cell);
    w->hoz = (float)(-0.5 * w->hnz * cell);
    const size_t n = (size_t)d->capacity;
    w->keys = (uint32_t*)calloc(n, 4); w->vals = (uint32_t*)calloc(n, 4);
    w->keys_sorted = (uint32_t*)calloc(n, 4); w->vals_sorted = (uint32_t*)calloc(n, 4);
    w->tmp_k = (uint32_t*)calloc(n, 4); w->tmp_v = (uint32_t*)calloc(n, 4);
    w->bstart = (int32_t*)calloc((size_t)w->hbuckets, 4);
    w->bend = (int32_t*)calloc((size_t)w->hbuckets, 4);
    w->fx = (double*)calloc(n, 8); w->fy = (double*)calloc(n, 8); w->fz = (double*)calloc(n, 8);
    w->fscale = (double*)calloc(n, 8); w->vscale = (double*)calloc(n, 8); w->pscale = (double*)calloc(n, 8);
    w->co2_demand = (uint64_t*)calloc(w->g[AGB_FIELD_CO2].enabled ? (size_t)w->g[AGB_FIELD_CO2].count : 1, 8);
    w->scan_flags = (int32_t*)calloc(n, 4); w->prefix = (int32_t*)calloc(n, 4);
    w->compact_src = (int32_t*)calloc(n, 4); w->scratch = calloc(n, 8);
    if (!w->keys || !w->vals || !w->keys_sorted || !w->vals_sorted || !w->tmp_k || !w->tmp_v ||
        !w->bstart || !w->bend || !w->fx || !w->fy || !w->fz || !w->co2_demand ||
        !w->fscale || !w->vscale || !w->pscale ||
        !w->scan_flags || !w->prefix || !w->compact_src || !w->scratch) {
        orc_world_destroy(w);
        return AGB_OUT_OF_MEMORY;
    }
    w->physics_rate = d->physics_rate;
    w->biology_rate = d->biology_rate;
    *out = w;
    return 0;
}

int orc_world_set_clock(orc_world* w, double p, double b) {   /* world_set_clock, step.cu:206-215 */
    w->physics_rate = p < AGB_CLOCK_PHYSICS_MIN ? AGB_CLOCK_PHYSICS_MIN
                    : (p > AGB_CLOCK_PHYSICS_MAX ? AGB_CLOCK_PHYSICS_MAX : p);
    w->biology_rate = b < AGB_CLOCK_BIOLOGY_MIN ? AGB_CLOCK_BIOLOGY_MIN
                    : (b > AGB_CLOCK_BIOLOGY_MAX ? AGB_CLOCK_BIOLOGY_MAX : b);
    return 0;
}

int orc_world_import_cells(orc_world* w, const agb_cells* src, int32_t count, uint64_t next_id) {
    if (count < 0 || count > w->capacity) return AGB_CAPACITY_EXCEEDED;
    size_t sz[25]; void* p[25]; void* h[25];
    soa_sizes(sz); soa_ptrs(&w->c, p); host_ptrs(src, h);
    for (int k = 0; k < 25; ++k)
        if (h[k]) memcpy(*(void**)p[k], h[k], sz[k] * (size_t)count);
    w->count = count;
    w->next_id = next_id;
    return 0;
}

int orc_world_export_cells(orc_world* w, agb_cells* dst, int32_t max_count, int32_t* count,
                           uint64_t* next_id) {
    const int32_t n = w->count < max_count ? w->count : max_count;
    size_t sz[25]; void* p[25]; void* h[25];
    soa_sizes(sz); soa_ptrs(&w->c, p); host_ptrs(dst, h);
    for (int k = 0; k < 25; ++k)
        if (h[k] && n > 0) memcpy(h[k], *(void**)p[k], sz[k] * (size_t)n);
    if (count) *count = w->count;
    if (next_id) *next_id = w->next_id;
    return 0;
}

int orc_world_import_field(orc_world* w, int32_t f, const float* src) {
    if (f < 0 || f >= AGB_FIELD_COUNT || !w->g[f].enabled) return AGB_INVALID_ARGUMENT;
    memcpy(w->g[f].value, src, sizeof(float) * (size_t)w->g[f].count);
    return 0;
}
int orc_world_export_field(orc_world* w, int32_t f, float* dst) {
    if (f < 0 || f >= AGB_FIELD_COUNT || !w->g[f].enabled) return AGB_INVALID_ARGUMENT;
    memcpy(dst, w->g[f].value, sizeof(float) * (size_t)w->g[f].count);
    return 0;
}
/* world_apply_brush (src/sim/step.cu:80-89) over grid_brush and brush_kernel
 * (src/fields/diffuse.cu:62-89): value += amount * (1 - t^2)^2, t = r / radius, for
 * voxel centres within radius of (x, y). EXTENSION: a 3-D grid takes the disc on
 * every z plane; non-finite arguments and absent fields are rejected. */
int orc_world_apply_brush(orc_world* w, int32_t kind, double x, double y, double radius, double strength) {
    int32_t f;
    double amount = strength;
    switch (kind) {
        case AGB_BRUSH_HEAT: f = AGB_FIELD_TEMPERATURE; break;
        case AGB_BRUSH_CHILL: f = AGB_FIELD_TEMPERATURE; amount = -strength; break;
        case AGB_BRUSH_INJECT_CO2: f = AGB_FIELD_CO2; break;
        case AGB_BRUSH_INJECT_N2: f = AGB_FIELD_N2; break;
        default: return AGB_INVALID_ARGUMENT;
    }
    if (!isfinite(x) || !isfinite(y) || !isfinite(radius) || !isfinite(strength)) return AGB_INVALID_ARGUMENT;
    grid* g = &w->g[f];
    if (!g->enabled) return AGB_INVALID_ARGUMENT;
    if (radius <= 0.0) return 0;
    const float dx = g->dxf, cx = (float)x, cy = (float)y, rad = (float)radius, amt = (float)amount;
    const float hx = 0.5f * g->nx * dx, hy = 0.5f * g->ny * dx;
    for (int32_t z = 0; z < g->nz; ++z)
        for (int32_t j = 0; j < g->ny; ++j)
            for (int32_t i = 0; i < g->nx; ++i) {
                const float px = (i + 0.5f) * dx - hx;
                const float py = (j + 0.5f) * dx - hy;
                const float r = sqrtf((px - cx) * (px - cx) + (py - cy) * (py - cy));
                if (r > rad) continue;
                const float t = r / rad;
                const float q = (1.0f - t * t) * (1.0f - t * t);
                g->value[i + (int64_t)g->nx * (j + (int64_t)g->ny * z)] += amt * q;
            }
    return 0;
}

int orc_world_export_deposit(orc_world* w, int32_t f, uint64_t* dst) {
    if (f < 0 || f >= AGB_FIELD_COUNT || !w->g[f].enabled) return AGB_INVALID_ARGUMENT;
    memcpy(dst, w->g[f].deposit, sizeof(uint64_t) * (size_t)w->g[f].count);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Spawn: spawn_kernel, src/sim/cell_store.cu:42-130 (+ EXTENSION placements) */
/* ------------------------------------------------------------------------- */
static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

static double sample_charge(pcg32* r, const agb_spawn* p) {   /* cell_store.cu:33-40 */
    switch (p->charge_dist) {
        case AGB_DIST_UNIFORM: return uniform_range(r, p->charge_a, p->charge_b);
        case AGB_DIST_NORMAL: return p->charge_a + p->charge_b * gaussian(r);
        case AGB_DIST_LOGNORMAL: return exp(log(p->charge_a) + p->charge_b * gaussian(r));
        default: return p->charge_a;
    }
}

/* EXTENSION: the centre of cluster k, from its own stream keyed on (seed, k). */
static vec3 cluster_centre(uint64_t seed, int32_t k, double extent) {
    const uint64_t id = 0xC1A5C1A5ull + (uint64_t)k;
    pcg32 r = cell_rng(cell_rng_init(seed ^ 0x5EEDC1A5ull, id), id);
    const double h = 0.5 * extent;
    const double x = uniform_range(&r, -h, h);
    const double y = uniform_range(&r, -h, h);
    const double z = uniform_range(&r, -h, h);
    return v3(x, y, z);
}

/* cell_store_spawn (src/sim/cell_store.cu:42-130, 250-280) with its seed argument. */
int orc_world_spawn_seeded(orc_world* w, const agb_spawn* p, uint64_t seed) {
    if (p->count <= 0) return 0;
    if (w->count + p->count > w->capacity) return AGB_CAPACITY_EXCEEDED;   /* cell_store.cu:264-265 */
    if (p->placement == AGB_PLACE_CLUSTERS && p->clusters <= 0) return AGB_INVALID_ARGUMENT;
    const double cw = w->d.chamber_w, ch = w->d.chamber_h, cd = w->d.chamber_d;
    const double a = AGB_CELL_RADIUS;
    soa* v = &w->c;
    for (int32_t i = 0; i < p->count; ++i) {
        const int32_t slot = w->count + i;
        const uint64_t id = w->next_id + (uint64_t)i;
        const uint64_t state = cell_rng_init(seed, id);
        pcg32 r = cell_rng(state, id);
        double x = 0.0, y = 0.0, z = 0.0;
        int z_done = 0;
        switch (p->placement) {
            case AGB_PLACE_GAUSSIAN: {
                double gx, gy;
                gaussian_pair(&r, &gx, &gy);
                x = p->place_x + p->place_radius * gx;
                y = p->place_y + p->place_radius * gy;
                break;
            }
            case AGB_PLACE_DISC: {
                const double rad = p->place_radius * sqrt(uniform01d(&r));
                const double ang = uniform_range(&r, 0.0, AGB_TWO_PI);
                x = p->place_x + rad * cos(ang);
                y = p->place_y + rad * sin(ang);
                break;
            }
            case AGB_PLACE_GRID: {
                const int side = (int)ceil(sqrt((double)p->count));
                const int gx = i % side, gy = i / side;
                x = ((double)gx / side - 0.5) * cw * 0.98;
                y = ((double)gy / side - 0.5) * ch * 0.98;
                break;
            }
            case AGB_PLACE_SLAB_X:
                x = uniform_range(&r, p->place_x - p->place_radius, p->place_x + p->place_radius);
                y = uniform_range(&r, -0.5 * ch, 0.5 * ch);
                break;
            case AGB_PLACE_CLUSTERS: {
                int32_t k = (int32_t)(uniform01d(&r) * (double)p->clusters);
                if (k >= p->clusters) k = p->clusters - 1;
                const vec3 c0 = cluster_centre(seed, k, p->cluster_extent);
                double gx, gy, gz, gw;
                gaussian_pair(&r, &gx, &gy);
                gaussian_pair(&r, &gz, &gw);
                x = c0.x + p->place_radius * gx;
                y = c0.y + p->place_radius * gy;
                z = clampd(c0.z + p->place_radius * gz, -0.5 * cd + a, 0.5 * cd - a);
                z_done = 1;
                break;
            }
            default:
                x = uniform_range(&r, -0.5 * cw, 0.5 * cw);
                y = uniform_range(&r, -0.5 * ch, 0.5 * ch);
                break;
        }
        x = clampd(x, -0.5 * cw + a, 0.5 * cw - a);
        y = clampd(y, -0.5 * ch + a, 0.5 * ch - a);
        if (!z_done) z = uniform_range(&r, -0.5 * cd + a, 0.5 * cd - a);
        double charge = clampd(sample_charge(&r, p), 0.0, 1.0);
        if (p->charge_max > 0.0 && charge > p->charge_max) charge = p->charge_max;
        v->id[slot] = id;
        v->flags[slot] = AGB_FLAG_OCCUPIED | AGB_FLAG_ALIVE | (p->awake ? AGB_FLAG_AWAKE : 0u);
        v->death_cause[slot] = AGB_DEATH_NONE;
        v->x[slot] = x; v->y[slot] = y; v->z[slot] = z;
        v->vx[slot] = 0.0; v->vy[slot] = 0.0; v->vz[slot] = 0.0;
        v->energy[slot] = charge * AGB_CELL_ENERGY_MAX;
        v->temp_cell[slot] = (float)(p->awake ? AGB_CELL_TEMP_SETPOINT : AGB_AMBIENT_TEMP_DEFAULT);
        v->emit_power[slot] = 0.0f;
        double dx, dy, dz, dd;                             /* gaussian3, rng.cuh:111-117 */
        gaussian_pair(&r, &dx, &dy);
        gaussian_pair(&r, &dz, &dd);
        const vec3 dir = vnormalize(v3(dx, dy, dz));
        v->dir_x[slot] = (float)dir.x; v->dir_y[slot] = (float)dir.y; v->dir_z[slot] = (float)dir.z;
        v->biomass[slot] = AGB_CELL_MASS_DRY;
        v->co2_held[slot] = 0.0;
        v->age_s[slot] = 0.0f;
        v->rng_state[slot] = r.state;
        v->taxis_memory[slot] = 0.0f;
        v->run_timer[slot] = 0.0f;
        v->t_local[slot] = v->temp_cell[slot];
        v->irradiance[slot] = 0.0f;
        v->co2_local[slot] = 0.0f;
        v->n2_local[slot] = 0.0f;
    }
    w->count += p->count;
    w->next_id += (uint64_t)p->count;
    return 0;
}

int orc_world_spawn(orc_world* w, const agb_spawn* p) { return orc_world_spawn_seeded(w, p, w->d.seed); }

/* The primary light source, replaced between ticks (the emission stage reads it). */
int orc_world_set_light(orc_world* w, const agb_light* light) {
    w->d.light = *light;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Spatial hash: src/sim/hash.cuh:59-111, src/sim/hash.cu:15-38, 106-133      */
/* ------------------------------------------------------------------------- */
static int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

static void hash_coords(const orc_world* w, double x, double y, double z, int32_t* gx, int32_t* gy,
                        int32_t* gz) {                    /* hash.cuh:63-68 */
    *gx = clampi((int32_t)((x - w->hox) * w->hinv), 0, w->hnx - 1);
    *gy = clampi((int32_t)((y - w->hoy) * w->hinv), 0, w->hny - 1);
    *gz = clampi((int32_t)((z - w->hoz) * w->hinv), 0, w->hnz - 1);
}
static uint32_t hash_index(const orc_world* w, int32_t gx, int32_t gy, int32_t gz) {
    return (uint32_t)((gz * w->hny + gy) * w->hnx + gx);   /* hash.cuh:70-72 */
}

/* Stable LSD radix sort of (key, value) on the bits the bucket count needs;
 * identical output to CUB's stable SortPairs over all 32 bits. */
static void stable_sort_pairs(orc_world* w, int32_t n) {
    uint32_t bits = 0;
    while (bits < 32 && ((uint64_t)w->hbuckets >> bits) != 0) ++bits;
    uint32_t *ik = w->keys, *iv = w->vals, *ok = w->keys_sorted, *ov = w->vals_sorted;
    memcpy(ok, ik, 4 * (size_t)n); memcpy(ov, iv, 4 * (size_t)n);
    uint32_t *ak = ok, *av = ov, *bk = w->tmp_k, *bv = w->tmp_v;
    for (uint32_t shift = 0; shift < bits; shift += 8) {
        size_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int32_t i = 0; i < n; ++i) ++cnt[((ak[i] >> shift) & 255u) + 1];
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int32_t i = 0; i < n; ++i) {
            const size_t pos = cnt[(ak[i] >> shift) & 255u]++;
            bk[pos] = ak[i]; bv[pos] = av[i];
        }
        uint32_t* t = ak; ak = bk; bk = t; t = av; av = bv; bv = t;
    }
    if (ak != ok) { memcpy(ok, ak, 4 * (size_t)n); memcpy(ov, av, 4 * (size_t)n); }
}

static int hash_build(orc_world* w) {
    const int32_t n = w->count;
    if (n <= 0) return 0;                                  /* hash.cu:107 */
    memset(w->bstart, 0, 4 * (size_t)w->hbuckets);         /* hash.cu:110-113 */
    memset(w->bend, 0, 4 * (size_t)w->hbuckets);
    for (int32_t i = 0; i < n; ++i) {                      /* key_kernel, hash.cu:15-25 */
        w->vals[i] = (uint32_t)i;
        if (w->c.flags[i] & AGB_FLAG_OCCUPIED) {
            int32_t gx, gy, gz;
            hash_coords(w, w->c.x[i], w->c.y[i], w->c.z[i], &gx, &gy, &gz);
            w->keys[i] = hash_index(w, gx, gy, gz);
        } else {
            w->keys[i] = (uint32_t)w->hbuckets;
        }
    }
    stable_sort_pairs(w, n);                               /* hash.cu:125-126 */
    for (int32_t i = 0; i < n; ++i) {                      /* range_kernel, hash.cu:29-38 */
        const uint32_t k = w->keys_sorted[i];
        if (k >= (uint32_t)w->hbuckets) continue;
        if (i == 0 || w->keys_sorted[i - 1] != k) w->bstart[k] = i;
        if (i == n - 1 || w->keys_sorted[i + 1] != k) w->bend[k] = i + 1;
    }
    return 0;
}

/* ASTRO_FOR_EACH_NEIGHBOUR, hash.cuh:88-111, as an explicit iterator. */
typedef struct { int32_t gx, gy, gz, dz, dy, dx, k, e; } nbr_it;
static void nbr_begin(const orc_world* w, nbr_it* it, double px, double py, double pz) {
    hash_coords(w, px, py, pz, &it->gx, &it->gy, &it->gz);
    it->dz = -1; it->dy = -1; it->dx = -2; it->k = 0; it->e = 0;
}
static int nbr_next(const orc_world* w, nbr_it* it, int32_t* j) {
    for (;;) {
        if (it->k < it->e) { *j = (int32_t)w->vals_sorted[it->k++]; return 1; }
        if (++it->dx > 1) {
            it->dx = -1;
            if (++it->dy > 1) { it->dy = -1; if (++it->dz > 1) return 0; }
        }
        const int32_t cz = it->gz + it->dz, cy = it->gy + it->dy, cx = it->gx + it->dx;
        if (cz < 0 || cz >= w->hnz || cy < 0 || cy >= w->hny || cx < 0 || cx >= w->hnx) continue;
        const uint32_t b = hash_index(w, cx, cy, cz);
        it->k = w->bstart[b];
        it->e = w->bend[b];
    }
}

int orc_world_export_hash(orc_world* w, int32_t dims[4], uint32_t* ks, uint32_t* vs, int32_t* bs,
                          int32_t* be) {
    dims[0] = w->hnx; dims[1] = w->hny; dims[2] = w->hnz; dims[3] = w->hbuckets;
    if (ks) memcpy(ks, w->keys_sorted, 4 * (size_t)w->count);
    if (vs) memcpy(vs, w->vals_sorted, 4 * (size_t)w->count);
    if (bs) memcpy(bs, w->bstart, 4 * (size_t)w->hbuckets);
    if (be) memcpy(be, w->bend, 4 * (size_t)w->hbuckets);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Thermal: src/sim/thermal.cu:19-103, src/sim/thermal.cuh:51-86              */
/* ------------------------------------------------------------------------- */
static void thermal_cells(orc_world* w, grid* T, double dt_sub, double cap, double cond) {
    soa* v = &w->c;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int32_t i = 0; i < w->count; ++i) {               /* thermal_kernel, thermal.cu:19-71 */
        const uint32_t flags = v->flags[i];
        if (!(flags & AGB_FLAG_OCCUPIED)) continue;
        const float xf = (float)v->x[i], yf = (float)v->y[i], zf = (float)v->z[i];
        const int64_t idx = grid_nearest(T, xf, yf, zf);
        const float t_grid = T->value[idx];
        int awake = (flags & AGB_FLAG_AWAKE) != 0u;
        if (!awake && (double)t_grid >= AGB_CELL_TEMP_SETPOINT) {   /* should_ignite */
            awake = 1;
            v->flags[i] = flags | AGB_FLAG_AWAKE;
        }
        const double t_cell = awake ? AGB_CELL_TEMP_SETPOINT : (double)t_grid;
        v->temp_cell[i] = (float)t_cell;
        if (!awake || !(flags & AGB_FLAG_ALIVE)) continue;
        double e = 0.0;                                    /* lumped_exchange_energy, thermal.cuh:80-86 */
        if (cap > 0.0 && cond > 0.0) {
            const double relax = -expm1(-cond * dt_sub / cap);
            e = cap * (t_cell - (double)t_grid) * relax;
        }
        double energy = v->energy[i] - e;
        double moved = e;
        if (energy < 0.0) { moved = v->energy[i]; energy = 0.0; }
        else if (energy > AGB_CELL_ENERGY_MAX) { moved = v->energy[i] - AGB_CELL_ENERGY_MAX; energy = AGB_CELL_ENERGY_MAX; }
        v->energy[i] = energy;
        deposit_add(&T->deposit[idx], moved / cap, T->deposit_scale);
        if (energy <= 0.0) {
            v->flags[i] = v->flags[i] & ~AGB_FLAG_ALIVE;
            v->death_cause[i] = AGB_DEATH_STARVED;
            v->emit_power[i] = 0.0f;
        }
    }
}

static int thermal_step(orc_world* w, double dt) {       /* thermal_step, thermal.cu:75-103 */
    grid* T = &w->g[AGB_FIELD_TEMPERATURE];
    if (!T->enabled) return 0;
    const int32_t substeps = grid_substeps(T, dt);
    const double dt_sub = dt / substeps;
    const double cap = AGB_WATER_DENSITY * AGB_WATER_SPECIFIC_HEAT * T->dx * T->dx * T->dz_eff;
    const double cond = AGB_CONDUCTION_COEFF;
    const float coeff = grid_coeff(T, dt_sub);
    if (!coeff_stable(T, coeff)) return AGB_INVALID_ARGUMENT;
    for (int32_t s = 0; s < substeps; ++s) {
        if (w->count > 0 && w->d.thermal_enabled) {
            thermal_cells(w, T, dt_sub, cap, cond);
            grid_flush(T);
        }
        grid_pass(T, coeff);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Emission: src/sim/emission.cu:17-177, src/sim/emission.cuh:19-53           */
/* ------------------------------------------------------------------------- */
static double disc_overlap_fraction(double p, double a) {   /* emission.cuh:19-25 */
    if (p <= 0.0) return 1.0;
    if (p >= 2.0 * a) return 0.0;
    const double x = p / (2.0 * a);
    return (2.0 / AGB_PI) * (acos(x) - x * sqrt(1.0 - x * x));
}
static double shadow_fraction(vec3 self, vec3 other, vec3 L) {   /* emission.cuh:30-37 */
    const vec3 d = vsub(self, other);
    const double along = vdot(d, L);
    if (along <= 0.0) return 0.0;
    const double perp2 = vdot(d, d) - along * along;
    const double perp = perp2 > 0.0 ? sqrt(perp2) : 0.0;
    return disc_overlap_fraction(perp, AGB_CELL_RADIUS);
}
static double column_transmittance(double area, double face) {   /* emission.cuh:43-47 */
    if (face <= 0.0) return 1.0;
    const double t = 1.0 - area / face;
    return t > 0.0 ? t : 0.0;
}

/* Sweep axis: emission.cu:161-163 (x or y); EXTENSION: z when it dominates. */
static int light_axis(vec3 d, int* sign) {
    const double ax = fabs(d.x), ay = fabs(d.y), az = fabs(d.z);
    int axis = (ax >= ay) ? 0 : 1;
    if (az > ax && az > ay) axis = 2;
    const double c = axis == 0 ? d.x : (axis == 1 ? d.y : d.z);
    *sign = c >= 0.0 ? 1 : -1;
    return axis;
}

static void emission_step(orc_world* w, double dt) {
    grid* I = &w->g[AGB_FIELD_IRRADIANCE];
    if (!I->enabled) return;
    const agb_light* L = &w->d.light;
    const float source = L->enabled ? L->irradiance : 0.0f;
    const float ambient = L->ambient;
    if (source <= 0.0f && ambient <= 0.0f) return;         /* emission.cu:150 */
    const vec3 dir = vnormalize(v3(L->dir_x, L->dir_y, L->dir_z));
    memset(I->deposit, 0, sizeof(uint64_t) * (size_t)I->count);   /* clear_kernel */
    soa* v = &w->c;
    if (w->count > 0 && source > 0.0f) {                   /* occlusion_stamp_kernel, :17-27 */
        for (int32_t i = 0; i < w->count; ++i) {
            const uint32_t f = v->flags[i];
            if (!(f & AGB_FLAG_OCCUPIED)) continue;
            const double area = (f & AGB_FLAG_ALIVE) ? AGB_CELL_CROSS_SECTION
                                                     : AGB_CELL_CROSS_SECTION * (1.0 - AGB_CELL_ALBEDO_DEAD);
            const int64_t idx = grid_nearest(I, (float)v->x[i], (float)v->y[i], (float)v->z[i]);
            deposit_add(&I->deposit[idx], area, I->deposit_scale);
        }
    }
    int sign;
    const int axis = light_axis(dir, &sign);
    /* Face of one voxel across the sweep: emission.cu:164 (dx * chamber depth). */
    const double face = axis == 2 ? I->dx * I->dx : I->dx * I->dz_eff;
    const int32_t nx = I->nx, ny = I->ny, nz = I->nz;
    const int64_t plane = (int64_t)nx * ny;
    const int32_t len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? nx : plane);
    const int64_t lines = I->count / len;
    for (int64_t line = 0; line < lines; ++line) {         /* sweep_kernel, :37-53 */
        int64_t base;
        if (axis == 0) base = line * nx;
        else if (axis == 1) base = (line % nx) + (line / nx) * plane;
        else base = line;
        double t = 1.0;
        for (int32_t s = 0; s < len; ++s) {
            const int32_t step = sign > 0 ? s : (len - 1 - s);
            const int64_t idx = base + stride * step;
            I->value[idx] = (float)(source * t) + ambient;
            const double area = from_fixed(I->deposit[idx], I->deposit_scale);
            t *= column_transmittance(area, face);
        }
    }
    if (w->count <= 0) return;
    const unsigned char exact = w->d.occlusion_exact;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int32_t i = 0; i < w->count; ++i) {               /* feed_kernel, :81-115 */
        const uint32_t f = v->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        const vec3 pos = v3(v->x[i], v->y[i], v->z[i]);
        double directional = (double)grid_sample(I, (float)pos.x, (float)pos.y, (float)pos.z) - ambient;
        if (directional < 0.0) directional = 0.0;
        if (exact) {
            double open = 1.0;
            nbr_it it;
            int32_t j;
            nbr_begin(w, &it, pos.x, pos.y, pos.z);
            while (nbr_next(w, &it, &j)) {
                if (j != i && (v->flags[j] & AGB_FLAG_OCCUPIED) && (v->flags[j] & AGB_FLAG_ALIVE))
                    open *= (1.0 - shadow_fraction(pos, v3(v->x[j], v->y[j], v->z[j]), dir));
            }
            directional *= open;
        }
        v->irradiance[i] = (float)directional;
        const double gained = (directional * AGB_CELL_CROSS_SECTION + (double)ambient * AGB_CELL_SURFACE_AREA) * dt;
        double e = v->energy[i] + gained;
        if (e > AGB_CELL_ENERGY_MAX) e = AGB_CELL_ENERGY_MAX;
        v->energy[i] = e;
    }
}

/* ------------------------------------------------------------------------- */
/* Motion: src/sim/integrator.cu:20-177, src/sim/integrator.cuh:29-254        */
/* ------------------------------------------------------------------------- */
static double cell_mass(double biomass, double energy) {   /* integrator.cuh:42-44 */
    return biomass + energy / (AGB_C_LIGHT * AGB_C_LIGHT);
}
static double drag_coefficient(double t) {                /* integrator.cuh:29-37 */
    return 6.0 * AGB_PI * (AGB_VF_A * exp(AGB_VF_B / (t - AGB_VF_C))) * AGB_CELL_RADIUS;
}
static double ou_position_shape(double x) {               /* integrator.cuh:80-91 */
    if (x < 1.0e-2) {
        const double x3 = x * x * x;
        return x3 * (2.0 / 3.0 + x * (-0.5 + x * (7.0 / 30.0 + x * (-1.0 / 12.0))));
    }
    const double e = exp(-x);
    return 2.0 * x - 3.0 + 4.0 * e - e * e;
}
typedef struct { double e1, ome, inv_beta, s_rr, s_vv, s_rv; } ou_coef;
static ou_coef ou_coefficients(double mass, double gamma, double T, double dt) {   /* :103-121 */
    ou_coef c;
    const double beta = gamma / mass;
    const double x = beta * dt;
    c.ome = -expm1(-x);
    c.e1 = 1.0 - c.ome;
    c.inv_beta = 1.0 / beta;
    const double kTm = AGB_K_BOLTZ * T / mass;
    const double var_vv = kTm * (-expm1(-2.0 * x));
    const double var_rr = kTm * c.inv_beta * c.inv_beta * ou_position_shape(x);
    c.s_vv = sqrt(var_vv > 0.0 ? var_vv : 0.0);
    c.s_rr = sqrt(var_rr > 0.0 ? var_rr : 0.0);
    c.s_rv = kTm * c.inv_beta * c.ome * c.ome;
    return c;
}
static void ou_advance_axis(double* pos, double* vel, double force, double gamma, const ou_coef* c,
                            double dt, int noise, double z1, double z2) {   /* :128-154 */
    const double v_term = force / gamma;
    const double dpos = v_term * dt + (*vel - v_term) * c->ome * c->inv_beta;
    const double dvel = (v_term - *vel) * c->ome;
    double npos = *pos + dpos;
    double nvel = *vel + dvel;
    if (noise && c->s_rr > 0.0) {
        const double a = c->s_rv / c->s_rr;
        const double b2 = c->s_vv * c->s_vv - a * a;
        const double b = sqrt(b2 > 0.0 ? b2 : 0.0);
        npos += c->s_rr * z1;
        nvel += a * z1 + b * z2;
    } else if (noise) {
        nvel += c->s_vv * z2;
    }
    *pos = npos;
    *vel = nvel;
}
static int apply_boundary_axis(double* p, double* v, double half, double radius, int mode) {   /* :233-254 */
    const double lo = -half + radius;
    const double hi = half - radius;
    if (*p >= lo && *p <= hi) return 1;
    if (mode == AGB_WALL_PERIODIC) {
        const double span = 2.0 * half;
        for (int k = 0; k < 64 && *p < -half; ++k) *p += span;   /* bounded for non-finite input */
        for (int k = 0; k < 64 && *p > half; ++k) *p -= span;
        return 1;
    }
    if (mode == AGB_WALL_ABSORBING) return 0;
    *p = (*p < lo) ? lo : hi;
    *v = 0.0;
    return 1;
}

static void motion_step(orc_world* w, double dt) {        /* motion_step, integrator.cu:154-177 */
    soa* v = &w->c;
    const int32_t n = w->count;
    if (n <= 0) return;
    const grid *T = &w->g[AGB_FIELD_TEMPERATURE], *C = &w->g[AGB_FIELD_CO2], *N = &w->g[AGB_FIELD_N2];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int32_t i = 0; i < n; ++i) {                      /* field_sample_kernel, :20-30 */
        if (!(v->flags[i] & AGB_FLAG_OCCUPIED)) continue;
        const float x = (float)v->x[i], y = (float)v->y[i], z = (float)v->z[i];
        if (T->enabled) v->t_local[i] = grid_sample(T, x, y, z);
        if (C->enabled) v->co2_local[i] = grid_sample(C, x, y, z);
        if (N->enabled) v->n2_local[i] = grid_sample(N, x, y, z);
    }
    const double kc = AGB_CONTACT_STIFFNESS / w->physics_rate;
    const double kt = w->d.trap_stiffness / w->physics_rate;
    const double two_a = AGB_CELL_DIAMETER;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int32_t i = 0; i < n; ++i) {                      /* forces_kernel, :40-76 */
        const uint32_t flags = v->flags[i];
        if (!(flags & AGB_FLAG_OCCUPIED)) { w->fx[i] = w->fy[i] = w->fz[i] = w->fscale[i] = 0.0; continue; }
        const double mass = cell_mass(v->biomass[i], v->energy[i]);
        const int alive = (flags & AGB_FLAG_ALIVE) != 0u;
        const double emit = alive ? (double)v->emit_power[i] : 0.0;
        vec3 F = v3(0.0, 0.0, 0.0);                        /* cell_force, integrator.cuh:179-188 */
        const double wgt = -(mass - AGB_WATER_DENSITY * AGB_CELL_VOLUME) * AGB_G_ACCEL;
        if (w->d.gravity_axis == AGB_GRAVITY_Y) F.y += wgt; else F.z += wgt;
        const double thrust = emit / AGB_C_LIGHT;
        /* checker: summed term magnitudes; the buoyant weight is the difference
         * of the cell's weight and that of the water it displaces */
        double fs = (mass + AGB_WATER_DENSITY * AGB_CELL_VOLUME) * AGB_G_ACCEL + fabs(thrust);
        if (thrust != 0.0) {
            F.x -= (double)v->dir_x[i] * thrust;
            F.y -= (double)v->dir_y[i] * thrust;
            F.z -= (double)v->dir_z[i] * thrust;
        }
        if (w->d.contact_enabled) {
            const vec3 pos = v3(v->x[i], v->y[i], v->z[i]);
            nbr_it it;
            int32_t j;
            nbr_begin(w, &it, pos.x, pos.y, pos.z);
            while (nbr_next(w, &it, &j)) {
                if (j == i || !(v->flags[j] & AGB_FLAG_OCCUPIED)) continue;
                const vec3 d = vsub(pos, v3(v->x[j], v->y[j], v->z[j]));   /* contact_force, :210-219 */
                const double r2 = vdot(d, d);
                if (r2 >= two_a * two_a || r2 <= 0.0) continue;
                const double r = sqrt(r2);
                const double overlap = two_a - r;
                const double s = kc * overlap / r;
                F.x += d.x * s; F.y += d.y * s; F.z += d.z * s;
                fs += kc * two_a;                          /* a contact's force at full overlap */
            }
        }
        if (i == w->d.trap_slot) {                          /* trap_force, :195-197 */
            F.x += kt * (w->d.trap_x - v->x[i]);
            F.y += kt * (w->d.trap_y - v->y[i]);
            F.z += 0.0;
            fs += fabs(kt * (w->d.trap_x - v->x[i])) + fabs(kt * (w->d.trap_y - v->y[i]));
        }
        w->fx[i] = F.x; w->fy[i] = F.y; w->fz[i] = F.z;
        w->fscale[i] = fs;
    }
    const double a = AGB_CELL_RADIUS;
    const double hw = 0.5 * w->d.chamber_w, hh = 0.5 * w->d.chamber_h, hd = 0.5 * w->d.chamber_d;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int32_t i = 0; i < n; ++i) {                      /* integrate_kernel, :79-150 */
        const uint32_t flags = v->flags[i];
        if (!(flags & AGB_FLAG_OCCUPIED)) continue;
        const double t_local = (double)v->t_local[i];
        const double mass = cell_mass(v->biomass[i], v->energy[i]);
        const int awake = (flags & AGB_FLAG_AWAKE) != 0u;
        const double t_drag = awake ? AGB_CELL_TEMP_SETPOINT : t_local;
        double gamma = drag_coefficient(t_drag);
        double px = v->x[i], py = v->y[i], pz = v->z[i];
        double ux = v->vx[i], uy = v->vy[i], uz = v->vz[i];
        if (flags & AGB_FLAG_STUCK) gamma *= AGB_WALL_STUCK_DRAG_MULT;
        pcg32 rng = cell_rng(v->rng_state[i], v->id[i]);
        const ou_coef c = ou_coefficients(mass, gamma, t_drag, dt);   /* integrate_cell, :158-169 */
        double z1, z2, z3, z4, z5, z6;
        gaussian_pair(&rng, &z1, &z2);
        gaussian_pair(&rng, &z3, &z4);
        gaussian_pair(&rng, &z5, &z6);
        ou_advance_axis(&px, &ux, w->fx[i], gamma, &c, dt, w->d.thermal_noise, z1, z2);
        ou_advance_axis(&py, &uy, w->fy[i], gamma, &c, dt, w->d.thermal_noise, z3, z4);
        ou_advance_axis(&pz, &uz, w->fz[i], gamma, &c, dt, w->d.thermal_noise, z5, z6);
        {   /* checker: the largest summed term magnitude of any axis's velocity and
             * displacement, the force term taken at its own term scale */
            const double vt = w->fscale[i] / gamma;
            const double za[3] = {fabs(z1), fabs(z3), fabs(z5)}, zb[3] = {fabs(z2), fabs(z4), fabs(z6)};
            const double u0[3] = {fabs(v->vx[i]), fabs(v->vy[i]), fabs(v->vz[i])};
            double ra = 0.0, rb = 0.0;
            if (w->d.thermal_noise && c.s_rr > 0.0) {
                ra = c.s_rv / c.s_rr;
                const double b2 = c.s_vv * c.s_vv - ra * ra;
                rb = sqrt(b2 > 0.0 ? b2 : 0.0);
            } else if (w->d.thermal_noise) {
                rb = c.s_vv;
            }
            double vs = 0.0, ps = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double sv = u0[k] * c.e1 + vt * c.ome + ra * za[k] + rb * zb[k];
                const double sp = vt * dt + (u0[k] + vt) * c.ome * c.inv_beta +
                                  (w->d.thermal_noise ? c.s_rr * za[k] : 0.0);
                if (sv > vs) vs = sv;
                if (sp > ps) ps = sp;
            }
            w->vscale[i] = vs;
            w->pscale[i] = ps;
        }
        v->rng_state[i] = rng.state;
        int kept = apply_boundary_axis(&px, &ux, hw, a, w->d.boundary_x);
        kept = apply_boundary_axis(&py, &uy, hh, a, w->d.boundary_y) && kept;
        const double z_before = pz;
        apply_boundary_axis(&pz, &uz, hd, a, AGB_WALL_REFLECTING);
        const int touched = (pz != z_before);
        uint32_t nf = flags;
        if (w->d.adhesion_enabled) {
            if (touched && !(flags & AGB_FLAG_STUCK)) {
                pcg32 ar = cell_rng(v->rng_state[i], v->id[i]);
                const int sticks = uniform01d(&ar) < AGB_WALL_STICKINESS;
                v->rng_state[i] = ar.state;
                if (sticks) nf |= AGB_FLAG_STUCK;
            } else if (flags & AGB_FLAG_STUCK) {
                const double away = (pz < 0.0) ? w->fz[i] : -w->fz[i];
                if (away > AGB_WALL_RELEASE_FORCE) nf &= ~AGB_FLAG_STUCK;
            }
        }
        v->flags[i] = nf;
        if (!kept) {
            v->flags[i] = nf & ~AGB_FLAG_ALIVE;
            v->death_cause[i] = AGB_DEATH_CULLED;
            v->emit_power[i] = 0.0f;
        }
        v->x[i] = px; v->y[i] = py; v->z[i] = pz;
        v->vx[i] = ux; v->vy[i] = uy; v->vz[i] = uz;
        v->age_s[i] += (float)dt;
    }
}

int orc_world_export_forces(orc_world* w, double* fx, double* fy, double* fz) {
    const size_t b = sizeof(double) * (size_t)w->count;
    memcpy(fx, w->fx, b); memcpy(fy, w->fy, b); memcpy(fz, w->fz, b);
    return 0;
}

/* Checker-only: per cell, from the last motion stage, the sum of the magnitudes
 * of the terms its force is made of (the cell's weight and the displaced
 * water's, recoil, trap, and k * 2a for each contact: the force of that
 * contact at full overlap), and the largest summed
 * term magnitude of any axis's velocity and displacement update. A value that
 * is a sum of terms can be held to a relative bound of that sum, not of itself:
 * contact sums cancel. */
int orc_world_export_term_scales(orc_world* w, double* force, double* vel, double* disp) {
    const size_t b = sizeof(double) * (size_t)w->count;
    memcpy(force, w->fscale, b); memcpy(vel, w->vscale, b); memcpy(disp, w->pscale, b);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Lifecycle: src/sim/lifecycle.cu:26-294, src/sim/lifecycle.cuh:24-99;       */
/* compaction: src/sim/cell_store.cu:368-456                                  */
/* ------------------------------------------------------------------------- */
static double co2_uptake_rate(double c) {                 /* lifecycle.cuh:24-28 */
    if (c <= 0.0) return 0.0;
    return AGB_LIFE_CO2_UPTAKE_MAX * c / (c + AGB_LIFE_CO2_HALF_SATURATION);
}
static int ready_to_divide(const orc_world* w, int32_t i) {   /* lifecycle.cuh:33-36 (+ EXTENSION) */
    if (w->d.division_predicate == AGB_DIVIDE_ENERGY) return w->c.energy[i] >= w->d.division_energy;
    return w->c.co2_held[i] >= w->d.co2_mass_per_division;
}
static void division_axis(uint64_t did, double* ax, double* ay, double* az) {   /* lifecycle.cuh:87-99 */
    const uint64_t h = splitmix64(splitmix64(did));
    const double u = (double)(h >> 33) * (1.0 / 2147483648.0) - 1.0;
    const double phi = (double)(h & 0xFFFFFFFFull) * (AGB_TWO_PI / 4294967296.0);
    const double s = sqrt(u * u < 1.0 ? 1.0 - u * u : 0.0);
    *ax = s * cos(phi);
    *ay = s * sin(phi);
    *az = u;
}

static void gather_all(orc_world* w, int32_t live) {      /* compact_field x 25, cell_store.cu:402-456 */
    size_t sz[25]; void* p[25];
    soa_sizes(sz); soa_ptrs(&w->c, p);
    unsigned char* sc = (unsigned char*)w->scratch;
    for (int k = 0; k < 25; ++k) {
        unsigned char* arr = *(unsigned char**)p[k];
        for (int32_t o = 0; o < live; ++o)
            memcpy(sc + sz[k] * (size_t)o, arr + sz[k] * (size_t)w->compact_src[o], sz[k]);
        memcpy(arr, sc, sz[k] * (size_t)live);
    }
}

static int compact(orc_world* w) {                        /* cell_store_compact, cell_store.cu:414-456 */
    const int32_t cnt = w->count;
    if (cnt <= 0) return 0;
    int32_t run = 0;
    for (int32_t i = 0; i < cnt; ++i) {
        const uint32_t f = w->c.flags[i];
        const int32_t keep = ((f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE)) ? 1 : 0;
        if (keep) w->compact_src[run] = i;
        run += keep;
    }
    const int32_t live = run;
    if (live >= cnt) return 0;
    if (live > 0) gather_all(w, live);
    double* sc[3] = {w->fscale, w->vscale, w->pscale};   /* checker arrays follow their cells */
    double* tmp = (double*)w->scratch;
    for (int k = 0; k < 3; ++k) {
        for (int32_t i = 0; i < live; ++i) tmp[i] = sc[k][w->compact_src[i]];
        memcpy(sc[k], tmp, sizeof(double) * (size_t)live);
    }
    w->count = live;
    return 0;
}

static void lifecycle_step(orc_world* w, double dt) {    /* lifecycle_step, lifecycle.cu:208-294 */
    soa* v = &w->c;
    const int32_t n = w->count;
    if (n <= 0) return;
    const double dt_bio = dt * w->biology_rate;
    grid* C = &w->g[AGB_FIELD_CO2];
    if (C->enabled) {
        const double gv = C->dx * C->dx * C->dz_eff;
        memset(w->co2_demand, 0, sizeof(uint64_t) * (size_t)C->count);   /* clear_u64_kernel */
        for (int32_t i = 0; i < n; ++i) {                  /* demand_kernel, :41-52 */
            const uint32_t f = v->flags[i];
            if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
            const int64_t idx = grid_nearest(C, (float)v->x[i], (float)v->y[i], (float)v->z[i]);
            const double want = co2_uptake_rate((double)C->value[idx]) * dt_bio;
            if (want <= 0.0) continue;
            deposit_add(&w->co2_demand[idx], want / gv, C->deposit_scale);
        }
        for (int32_t i = 0; i < n; ++i) {                  /* uptake_kernel, :62-86 */
            const uint32_t f = v->flags[i];
            if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
            const int64_t idx = grid_nearest(C, (float)v->x[i], (float)v->y[i], (float)v->z[i]);
            const double want = co2_uptake_rate((double)C->value[idx]) * dt_bio;
            if (want <= 0.0) continue;
            const double asked = from_fixed(w->co2_demand[idx], C->deposit_scale);
            const double available = (double)C->value[idx];
            double taken = want;
            if (asked > available && asked > 0.0) taken = want * (available / asked);
            if (taken <= 0.0) continue;
            v->co2_held[i] += taken;
            deposit_add(&C->deposit[idx], -taken / gv, C->deposit_scale);
        }
        grid_flush(C);                                     /* lifecycle.cu:235 */
    }
    for (int32_t i = 0; i < n; ++i) {                      /* death_kernel, :100-112 */
        const uint32_t f = v->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        if (!((double)v->t_local[i] > AGB_CELL_LETHAL_TEMP)) continue;
        v->flags[i] = f & ~AGB_FLAG_ALIVE;
        v->death_cause[i] = AGB_DEATH_OVERHEATED;
        v->emit_power[i] = 0.0f;
        v->energy[i] = w->d.store_disposition == AGB_STORE_RETAIN ? v->energy[i] : 0.0;   /* corpse_energy */
    }
    int32_t births = 0, deads = 0;
    for (int32_t i = 0; i < n; ++i) {                      /* mark_kernel, :119-135 */
        const uint32_t f = v->flags[i];
        const int occ = (f & AGB_FLAG_OCCUPIED) != 0u, alive = (f & AGB_FLAG_ALIVE) != 0u;
        const int div = occ && alive && ready_to_divide(w, i);
        w->scan_flags[i] = div;
        births += div;
        deads += (occ && !alive);
    }
    const int32_t new_deaths = deads - w->dead_slots_prev;
    if (new_deaths > 0) w->deaths_total += new_deaths;
    if (births > 0) {
        int32_t run = 0;                                   /* ExclusiveSum, :269-270 */
        for (int32_t i = 0; i < n; ++i) { w->prefix[i] = run; run += w->scan_flags[i]; }
        const int32_t base = n;
        if (base + births > w->capacity) births = w->capacity - base;
        if (births > 0) {
            const uint64_t first_id = w->next_id;
            const double a = AGB_CELL_RADIUS;
            const double hx = 0.5 * w->d.chamber_w - a, hy = 0.5 * w->d.chamber_h - a,
                         hz = 0.5 * w->d.chamber_d - a;
            for (int32_t i = 0; i < n; ++i) {              /* divide_kernel, :140-204 */
                const uint32_t f = v->flags[i];
                if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
                if (!ready_to_divide(w, i)) continue;
                const int32_t slot = base + w->prefix[i];
                if (slot >= w->capacity) continue;
                const uint64_t did = first_id + (uint64_t)w->prefix[i];
                const double half0 = 0.5 * (v->energy[i] - AGB_LIFE_DIVISION_ENERGY_COST);
                const double half = half0 > 0.0 ? half0 : 0.0;
                v->energy[i] = half;
                v->energy[slot] = half;
                v->co2_held[i] = 0.0;
                v->co2_held[slot] = 0.0;
                v->biomass[slot] = AGB_CELL_MASS_DRY;
                double ax, ay, az;
                division_axis(did, &ax, &ay, &az);
                v->x[slot] = v->x[i] + a * ax; v->x[i] -= a * ax;
                v->y[slot] = v->y[i] + a * ay; v->y[i] -= a * ay;
                v->z[slot] = v->z[i] + a * az; v->z[i] -= a * az;
                v->x[slot] = clampd(v->x[slot], -hx, hx);
                v->y[slot] = clampd(v->y[slot], -hy, hy);
                v->z[slot] = clampd(v->z[slot], -hz, hz);
                v->x[i] = clampd(v->x[i], -hx, hx);
                v->y[i] = clampd(v->y[i], -hy, hy);
                v->z[i] = clampd(v->z[i], -hz, hz);
                v->vx[slot] = v->vx[i]; v->vy[slot] = v->vy[i]; v->vz[slot] = v->vz[i];
                w->fscale[slot] = w->fscale[i]; w->vscale[slot] = w->vscale[i]; w->pscale[slot] = w->pscale[i];
                v->id[slot] = did;
                v->flags[slot] = v->flags[i];
                v->death_cause[slot] = AGB_DEATH_NONE;
                v->temp_cell[slot] = v->temp_cell[i];
                v->emit_power[slot] = 0.0f;
                v->dir_x[slot] = v->dir_x[i]; v->dir_y[slot] = v->dir_y[i]; v->dir_z[slot] = v->dir_z[i];
                v->age_s[slot] = 0.0f;
                v->rng_state[slot] = pcg_split(v->rng_state[i], did);
                v->taxis_memory[slot] = 0.0f;
                v->run_timer[slot] = 0.0f;
                v->t_local[slot] = v->t_local[i];
                v->irradiance[slot] = 0.0f;
                v->co2_local[slot] = v->co2_local[i];
                v->n2_local[slot] = v->n2_local[i];
            }
            w->divisions_this_window += births;
            w->next_id += (uint64_t)births;
            w->count += births;
        }
    }
    /* Compaction (lifecycle.cu:289-293); EXTENSION: only on every compaction_period-th tick. */
    const int32_t period = w->d.compaction_period > 0 ? w->d.compaction_period : 1;
    int compacted = 0;
    if (w->d.compaction_enabled && deads > 0 && ((w->tick + 1) % (uint64_t)period) == 0) {
        compact(w);
        compacted = 1;
    }
    w->dead_slots_prev = compacted ? 0 : deads;
}

/* ------------------------------------------------------------------------- */
/* Taxis: src/sim/taxis.cu:13-85, src/sim/taxis.cuh:31-143                   */
/* ------------------------------------------------------------------------- */
static vec3 vadd(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec3 vcross(vec3 a, vec3 b) {                      /* vec.cuh:39-41 */
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static vec3 any_perpendicular(vec3 v) {                   /* taxis.cuh:86-92 */
    const double ax = fabs(v.x), ay = fabs(v.y), az = fabs(v.z);
    const vec3 axis = (ax <= ay && ax <= az) ? v3(1.0, 0.0, 0.0) : (ay <= az) ? v3(0.0, 1.0, 0.0) : v3(0.0, 0.0, 1.0);
    return vnormalize(vcross(v, axis));
}
static vec3 rotate_by(vec3 h, double theta, double azimuth) {   /* taxis.cuh:95-100 */
    const vec3 u = any_perpendicular(h);
    const vec3 w = vcross(h, u);
    const vec3 perp = vadd(vscale(u, cos(azimuth)), vscale(w, sin(azimuth)));
    return vnormalize(vadd(vscale(h, cos(theta)), vscale(perp, sin(theta))));
}
static vec3 taxis_tumble(vec3 heading, pcg32* rng) {      /* taxis.cuh:109-118 */
    double theta = -AGB_TAXIS_TUMBLE_ANGLE_MEAN * log(1.0 - uniform01d(rng));
    if (theta > AGB_PI) theta = AGB_PI;
    const double azimuth = AGB_TWO_PI * uniform01d(rng);
    return rotate_by(vnormalize(heading), theta, azimuth);
}

static void taxis_step(orc_world* w, double dt) {
    const double max_power = w->d.max_emit_power > 0.0 ? w->d.max_emit_power : AGB_PETROVA_MAX_POWER;
    soa* v = &w->c;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < w->count; ++i) {
        const uint32_t f = v->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        if (!(f & AGB_FLAG_AWAKE)) { v->emit_power[i] = 0.0f; continue; }
        const double irr = (double)v->irradiance[i];
        const double co2 = (double)v->co2_local[i];
        const double charge = v->energy[i] / AGB_CELL_ENERGY_MAX;
        const int dark = irr < AGB_TAXIS_DARK_THRESHOLD, co2_here = co2 > 0.0;   /* taxis.cuh:56-62 */
        int state = 0;
        if (dark && !co2_here) state = 0;
        else if (!dark && charge < AGB_TAXIS_SEEK_FEED_BELOW) state = 1;
        else if (charge > AGB_TAXIS_SEEK_BREED_ABOVE && co2_here) state = 2;
        if (state == 0) {
            v->emit_power[i] = 0.0f;
            v->run_timer[i] = 0.0f;
            v->taxis_memory[i] = 0.0f;
            continue;
        }
        const double signal = state == 1 ? irr : co2;
        const double delta = signal - (double)v->taxis_memory[i];
        const double alpha = 1.0 - exp(-dt / AGB_TAXIS_MEMORY_TIME);       /* taxis.cuh:38-41 */
        v->taxis_memory[i] = (float)((double)v->taxis_memory[i] + alpha * (signal - (double)v->taxis_memory[i]));
        vec3 heading = v3(-(double)v->dir_x[i], -(double)v->dir_y[i], -(double)v->dir_z[i]);
        double run = (double)v->run_timer[i] + dt;
        if (delta <= 0.0 || run >= AGB_TAXIS_RUN_MAX) {
            pcg32 rng = cell_rng(v->rng_state[i], v->id[i]);
            heading = taxis_tumble(heading, &rng);
            v->rng_state[i] = rng.state;
            run = 0.0;
        }
        v->run_timer[i] = (float)run;
        const vec3 axis = vscale(vnormalize(heading), -1.0);           /* taxis_emit_dir */
        v->dir_x[i] = (float)axis.x;
        v->dir_y[i] = (float)axis.y;
        v->dir_z[i] = (float)axis.z;
        double p = 0.0;                                                 /* taxis.cuh:136-141 */
        if (v->energy[i] > 0.0) {
            const double avail = dt > 0.0 ? v->energy[i] / dt : 0.0;
            p = max_power < avail ? max_power : avail;
        }
        v->emit_power[i] = (float)p;
        v->energy[i] -= p * dt;
    }
}

/* ------------------------------------------------------------------------- */
/* Tick: world_step, src/sim/step.cu:109-184                                  */
/* ------------------------------------------------------------------------- */
static int slow_fields(orc_world* w, double dt) {         /* step.cu:168-171 */
    grid_flush(&w->g[AGB_FIELD_CO2]);
    grid_flush(&w->g[AGB_FIELD_N2]);
    int rc = grid_diffuse(&w->g[AGB_FIELD_CO2], dt);
    if (rc) return rc;
    return grid_diffuse(&w->g[AGB_FIELD_N2], dt);
}

/* flash_step / flash_kernel (src/sim/flash.cu:31-67): while armed, every awake
 * live cell discharges power * dt of its store at full rate, emit_power 0, the
 * photon impulse (-z) and the energy into the audit in fixed point. */
static void flash_step(orc_world* w, double dt) {
    if (!w->flash_active) return;
    soa* v = &w->c;
    for (int32_t i = 0; i < w->count; ++i) {
        const uint32_t f = v->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE) || !(f & AGB_FLAG_AWAKE)) continue;
        const double e = v->energy[i];
        v->emit_power[i] = 0.0f;
        if (e <= 0.0) continue;
        double de = w->flash_power * dt;
        if (de > e) de = e;
        v->energy[i] = e - de;
        const double imp = de / AGB_C_LIGHT;
        w->flash_accum[2] += (uint64_t)llround(-imp * AGB_FLASH_IMPULSE_SCALE);
        w->flash_accum[3] += (uint64_t)llround(de * AGB_FLASH_ENERGY_SCALE);
    }
}

/* ------------------------------------------------------------------------- */
/* Taumoeba, the predator: src/sim/predation.cu, src/sim/predation.cuh        */
/* ------------------------------------------------------------------------- */
static double water_viscosity(double t) { return AGB_VF_A * exp(AGB_VF_B / (t - AGB_VF_C)); }   /* integrator.cuh:29-31 */
static void gaussian3(pcg32* r, double* x, double* y, double* z) {   /* rng.cuh:111-117 */
    double a, b, c, d;
    gaussian_pair(r, &a, &b);
    gaussian_pair(r, &c, &d);
    (void)d;
    *x = a; *y = b; *z = c;
}

/* spawn_kernel + taumoeba_spawn (predation.cu:33-74, 420-432). */
int orc_world_spawn_taumoeba(orc_world* w, int32_t count, uint64_t seed) {
    if (count <= 0) return 0;
    if (w->tau_count + count > w->tau_capacity) return AGB_CAPACITY_EXCEEDED;
    tau_soa* t = &w->t;
    const double a = AGB_TAU_RADIUS;
    for (int32_t i = 0; i < count; ++i) {
        const int32_t slot = w->tau_count + i;
        const uint64_t id = w->tau_next_id + (uint64_t)i;
        pcg32 r = cell_rng(cell_rng_init(splitmix64(seed), id), id);
        t->x[slot] = uniform_range(&r, -0.5 * w->d.chamber_w + a, 0.5 * w->d.chamber_w - a);
        t->y[slot] = uniform_range(&r, -0.5 * w->d.chamber_h + a, 0.5 * w->d.chamber_h - a);
        t->z[slot] = uniform_range(&r, -0.5 * w->d.chamber_d + a, 0.5 * w->d.chamber_d - a);
        t->vx[slot] = 0.0; t->vy[slot] = 0.0; t->vz[slot] = 0.0;
        double dx, dy, dz;
        gaussian3(&r, &dx, &dy, &dz);
        const vec3 dir = vnormalize(v3(dx, dy, dz));
        t->dir_x[slot] = (float)dir.x; t->dir_y[slot] = (float)dir.y; t->dir_z[slot] = (float)dir.z;
        t->id[slot] = id;
        t->flags[slot] = AGB_FLAG_OCCUPIED | AGB_FLAG_ALIVE;
        t->biomass[slot] = AGB_TAU_MASS_DRY;
        t->prey_biomass[slot] = 0.0;
        t->digest_timer[slot] = 0.0f;
        t->tolerance[slot] = (float)AGB_TAU_N2_TOLERANCE_INIT;
        t->generation[slot] = 0u;
        t->rng_state[slot] = r.state;
        t->density_ema[slot] = 0.0f;
        t->run_timer[slot] = 0.0f;
        t->target[slot] = -1;
    }
    w->tau_count += count;
    w->tau_next_id += (uint64_t)count;
    return 0;
}

/* predation_step (predation.cu:434-484): hunt, resolve, nitrogen, division,
 * compaction, each pass over the predators in slot order. */
static void predation_step(orc_world* w, double dt) {
    const int32_t n = w->tau_count;
    if (n <= 0) return;
    tau_soa* t = &w->t;
    soa* c = &w->c;
    const double dt_bio = dt * w->biology_rate;
    memset(w->claim, 0xFF, 8 * (size_t)w->capacity);
    const double t_amb = w->d.ambient_temp;
    const double gamma = 6.0 * AGB_PI * water_viscosity(t_amb) * AGB_TAU_RADIUS;   /* tau_drag */
    const ou_coef oc = ou_coefficients(AGB_TAU_MASS, gamma, t_amb, dt);
    const double rr = (AGB_TAU_RADIUS + AGB_CELL_RADIUS) * (AGB_TAU_RADIUS + AGB_CELL_RADIUS);
    for (int32_t i = 0; i < n; ++i) {                      /* hunt_kernel, predation.cu:80-158 */
        const uint32_t f = t->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        vec3 pos = v3(t->x[i], t->y[i], t->z[i]);
        const int digesting = t->digest_timer[i] > 0.0f;
        int prey_count = 0;
        int32_t prey = -1;
        int32_t gx, gy, gz;
        hash_coords(w, pos.x, pos.y, pos.z, &gx, &gy, &gz);
        for (int32_t dz = -1; dz <= 1; ++dz) {             /* ASTRO_FOR_EACH_NEIGHBOUR, hash.cuh:88-111 */
            const int32_t cz = gz + dz;
            if (cz < 0 || cz >= w->hnz) continue;
            for (int32_t dy = -1; dy <= 1; ++dy) {
                const int32_t cy = gy + dy;
                if (cy < 0 || cy >= w->hny) continue;
                for (int32_t dx = -1; dx <= 1; ++dx) {
                    const int32_t cx = gx + dx;
                    if (cx < 0 || cx >= w->hnx) continue;
                    const uint32_t b = hash_index(w, cx, cy, cz);
                    for (int32_t k = w->bstart[b]; k < w->bend[b]; ++k) {
                        const int32_t j = (int32_t)w->vals_sorted[k];
                        const uint32_t cf = c->flags[j];
                        if (!(cf & AGB_FLAG_OCCUPIED) || !(cf & AGB_FLAG_ALIVE)) continue;
                        ++prey_count;
                        const vec3 d = vsub(pos, v3(c->x[j], c->y[j], c->z[j]));
                        if (prey < 0 && vdot(d, d) < rr) prey = j;
                    }
                }
            }
        }
        if (!digesting && prey >= 0) {
            t->target[i] = prey;
            if (t->id[i] < w->claim[prey]) w->claim[prey] = t->id[i];
        } else {
            t->target[i] = -1;
        }
        pcg32 rng = cell_rng(t->rng_state[i], t->id[i]);
        float ema = t->density_ema[i];
        float run = t->run_timer[i];
        vec3 dir = v3(t->dir_x[i], t->dir_y[i], t->dir_z[i]);
        const double alpha = -expm1(-dt / AGB_TAXIS_MEMORY_TIME);   /* tau_should_tumble, predation.cuh:36-41 */
        const double delta = (double)(float)prey_count - (double)ema;
        ema = (float)(ema + alpha * delta);
        if (!(delta > 0.0 && run < AGB_TAXIS_RUN_MAX)) {
            double gx3, gy3, gz3;
            gaussian3(&rng, &gx3, &gy3, &gz3);
            dir = vnormalize(v3(gx3, gy3, gz3));
            run = 0.0f;
        } else {
            run += (float)dt;
        }
        t->density_ema[i] = ema;
        t->run_timer[i] = run;
        t->dir_x[i] = (float)dir.x; t->dir_y[i] = (float)dir.y; t->dir_z[i] = (float)dir.z;
        double vel[3] = {t->vx[i], t->vy[i], t->vz[i]};
        double z[6];
        gaussian_pair(&rng, &z[0], &z[1]);                 /* integrate_cell, integrator.cuh:159-169 */
        gaussian_pair(&rng, &z[2], &z[3]);
        gaussian_pair(&rng, &z[4], &z[5]);
        ou_advance_axis(&pos.x, &vel[0], dir.x * AGB_TAU_CRAWL_THRUST, gamma, &oc, dt, w->d.thermal_noise, z[0], z[1]);
        ou_advance_axis(&pos.y, &vel[1], dir.y * AGB_TAU_CRAWL_THRUST, gamma, &oc, dt, w->d.thermal_noise, z[2], z[3]);
        ou_advance_axis(&pos.z, &vel[2], dir.z * AGB_TAU_CRAWL_THRUST, gamma, &oc, dt, w->d.thermal_noise, z[4], z[5]);
        t->rng_state[i] = rng.state;
        apply_boundary_axis(&pos.x, &vel[0], 0.5 * w->d.chamber_w, AGB_TAU_RADIUS, w->d.boundary_x);
        apply_boundary_axis(&pos.y, &vel[1], 0.5 * w->d.chamber_h, AGB_TAU_RADIUS, w->d.boundary_y);
        apply_boundary_axis(&pos.z, &vel[2], 0.5 * w->d.chamber_d, AGB_TAU_RADIUS, AGB_WALL_REFLECTING);
        t->x[i] = pos.x; t->y[i] = pos.y; t->z[i] = pos.z;
        t->vx[i] = vel[0]; t->vy[i] = vel[1]; t->vz[i] = vel[2];
        if (digesting) {
            float dg = t->digest_timer[i] - (float)dt_bio;
            if (dg <= 0.0f) {
                t->biomass[i] += t->prey_biomass[i] * AGB_TAU_BIOMASS_YIELD;
                t->prey_biomass[i] = 0.0;
                dg = 0.0f;
            }
            t->digest_timer[i] = dg;
        }
    }
    for (int32_t i = 0; i < n; ++i) {                      /* resolve_kernel, predation.cu:160-182 */
        const int32_t prey = t->target[i];
        if (prey < 0 || w->claim[prey] != t->id[i]) continue;
        const uint32_t cf = c->flags[prey];
        if (!(cf & AGB_FLAG_OCCUPIED) || !(cf & AGB_FLAG_ALIVE)) continue;
        c->flags[prey] = cf & ~AGB_FLAG_ALIVE;
        c->death_cause[prey] = AGB_DEATH_PREDATED;
        c->emit_power[prey] = 0.0f;
        c->energy[prey] = w->d.store_disposition == AGB_STORE_RETAIN ? c->energy[prey] : 0.0;   /* corpse_energy */
        t->digest_timer[i] = (float)AGB_TAU_DIGEST_TIME;
        t->prey_biomass[i] = c->biomass[prey];
    }
    const grid* n2 = &w->g[AGB_FIELD_N2];
    for (int32_t i = 0; i < n; ++i) {                      /* nitrogen_kernel, predation.cu:189-205 */
        const uint32_t f = t->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        pcg32 rng = cell_rng(t->rng_state[i], t->id[i]);
        const double u = uniform01d(&rng);
        t->rng_state[i] = rng.state;
        const double n2_local = n2->enabled ? (double)grid_sample(n2, (float)t->x[i], (float)t->y[i], (float)t->z[i]) : 0.0;
        const double thr = AGB_TAU_N2_LETHAL_CONC * (1.0 + (double)t->tolerance[i] * AGB_TAU_N2_TOLERANCE_K);
        const double h = n2_local - thr;
        const double hazard = h > 0.0 ? h : 0.0;
        if (u < -expm1(-hazard * AGB_TAU_N2_HAZARD_RATE * dt_bio)) t->flags[i] = f & ~AGB_FLAG_ALIVE;
    }
    /* tau_mark_kernel + the prefix sum + tau_divide_kernel (predation.cu:211-284, 458-477) */
    int32_t births = 0, deads = 0;
    for (int32_t i = 0; i < n; ++i) {
        const uint32_t f = t->flags[i];
        const int occ = (f & AGB_FLAG_OCCUPIED) != 0u, alive = (f & AGB_FLAG_ALIVE) != 0u;
        if (occ && !alive) ++deads;
        if (!(occ && alive) || !(t->biomass[i] >= AGB_TAU_DIVIDE_BIOMASS)) continue;
        const int32_t pre = births++;
        const int32_t slot = n + pre;
        if (slot >= w->tau_capacity) continue;
        const uint64_t did = w->tau_next_id + (uint64_t)pre;
        const double half = 0.5 * t->biomass[i];
        t->biomass[i] = half;
        t->biomass[slot] = half;
        pcg32 dr = cell_rng(pcg_split(t->rng_state[i], did), did);
        const double mutation = gaussian(&dr);
        double tol = (double)t->tolerance[i] + AGB_TAU_MUTATION_SIGMA * mutation;
        tol = tol < 0.0 ? 0.0 : (tol > 1.0 ? 1.0 : tol);
        t->tolerance[slot] = (float)tol;
        t->rng_state[slot] = dr.state;
        t->generation[slot] = t->generation[i] + 1u;
        double ax, ay, az;
        division_axis(did, &ax, &ay, &az);
        const double a = AGB_TAU_RADIUS;
        t->x[slot] = t->x[i] + a * ax;  t->x[i] -= a * ax;
        t->y[slot] = t->y[i] + a * ay;  t->y[i] -= a * ay;
        t->z[slot] = t->z[i] + a * az;  t->z[i] -= a * az;
        const double hx = 0.5 * w->d.chamber_w - a, hy = 0.5 * w->d.chamber_h - a, hz = 0.5 * w->d.chamber_d - a;
        t->x[slot] = clampd(t->x[slot], -hx, hx); t->y[slot] = clampd(t->y[slot], -hy, hy);
        t->z[slot] = clampd(t->z[slot], -hz, hz);
        t->x[i] = clampd(t->x[i], -hx, hx); t->y[i] = clampd(t->y[i], -hy, hy); t->z[i] = clampd(t->z[i], -hz, hz);
        t->id[slot] = did;
        t->flags[slot] = t->flags[i];
        t->vx[slot] = t->vx[i]; t->vy[slot] = t->vy[i]; t->vz[slot] = t->vz[i];
        t->dir_x[slot] = t->dir_x[i]; t->dir_y[slot] = t->dir_y[i]; t->dir_z[slot] = t->dir_z[i];
        t->prey_biomass[slot] = 0.0;
        t->digest_timer[slot] = 0.0f;
        t->density_ema[slot] = 0.0f;
        t->run_timer[slot] = 0.0f;
        t->target[slot] = -1;
    }
    if (n + births > w->tau_capacity) births = w->tau_capacity - n;
    if (births > 0) {
        w->tau_next_id += (uint64_t)births;
        w->tau_count += births;
    }
    if (w->d.tau_compaction_enabled && deads > 0) {         /* taumoeba_store_compact, predation.cu:486-521 */
        void** tp[20];
        tau_ptrs(t, tp);
        int32_t live = 0;
        for (int32_t i = 0; i < w->tau_count; ++i) {
            const uint32_t f = t->flags[i];
            if (!((f & AGB_FLAG_OCCUPIED) && (f & AGB_FLAG_ALIVE))) continue;
            if (live != i)
                for (int k = 0; k < 20; ++k) {
                    unsigned char* arr = (unsigned char*)*tp[k];
                    memmove(arr + TAU_SZ[k] * (size_t)live, arr + TAU_SZ[k] * (size_t)i, TAU_SZ[k]);
                }
            ++live;
        }
        w->tau_count = live;
    }
}

int orc_world_import_taumoeba(orc_world* w, const agb_taumoeba* src, int32_t count, uint64_t next_id) {
    if (count < 0 || count > w->tau_capacity) return AGB_CAPACITY_EXCEEDED;
    void* h[20] = {src->id, src->flags, src->x, src->y, src->z, src->vx, src->vy, src->vz, src->dir_x, src->dir_y,
                   src->dir_z, src->biomass, src->prey_biomass, src->digest_timer, src->tolerance, src->generation,
                   src->rng_state, src->density_ema, src->run_timer, src->target};
    void** tp[20];
    tau_ptrs(&w->t, tp);
    for (int k = 0; k < 20; ++k) {
        if (!h[k]) return AGB_INVALID_ARGUMENT;
        memcpy(*tp[k], h[k], TAU_SZ[k] * (size_t)count);
    }
    w->tau_count = count;
    w->tau_next_id = next_id;
    return 0;
}

int orc_world_export_taumoeba(orc_world* w, agb_taumoeba* dst, int32_t max_count, int32_t* count, uint64_t* next_id) {
    const int32_t n = w->tau_count < max_count ? w->tau_count : max_count;
    void* h[20] = {dst->id, dst->flags, dst->x, dst->y, dst->z, dst->vx, dst->vy, dst->vz, dst->dir_x, dst->dir_y,
                   dst->dir_z, dst->biomass, dst->prey_biomass, dst->digest_timer, dst->tolerance, dst->generation,
                   dst->rng_state, dst->density_ema, dst->run_timer, dst->target};
    void** tp[20];
    tau_ptrs(&w->t, tp);
    for (int k = 0; k < 20; ++k)
        if (h[k] && n > 0) memcpy(h[k], *tp[k], TAU_SZ[k] * (size_t)n);
    if (count) *count = w->tau_count;
    if (next_id) *next_id = w->tau_next_id;
    return 0;
}

int orc_world_set_flash(orc_world* w, int32_t active, double power) {
    w->flash_active = active != 0;
    w->flash_power = power > 0.0 ? power : AGB_PETROVA_FLASH_POWER;
    return 0;
}

/* world_flash_audit (src/sim/flash.cu:69-78). */
int orc_world_flash_audit(orc_world* w, double* impulse_ns, double* discharged_j) {
    const double ix = (double)(int64_t)w->flash_accum[0] / AGB_FLASH_IMPULSE_SCALE;
    const double iy = (double)(int64_t)w->flash_accum[1] / AGB_FLASH_IMPULSE_SCALE;
    const double iz = (double)(int64_t)w->flash_accum[2] / AGB_FLASH_IMPULSE_SCALE;
    *impulse_ns = sqrt(ix * ix + iy * iy + iz * iz);
    *discharged_j = (double)(int64_t)w->flash_accum[3] / AGB_FLASH_ENERGY_SCALE;
    return 0;
}

int orc_world_stage(orc_world* w, int32_t stage) {
    const double dt = AGB_DT_PHYSICS * w->physics_rate;
    switch (stage) {
        case AGB_STAGE_HASH: return hash_build(w);
        case AGB_STAGE_THERMAL: return thermal_step(w, dt);
        case AGB_STAGE_EMISSION: emission_step(w, dt); return 0;
        case AGB_STAGE_TAXIS: taxis_step(w, dt); return 0;
        case AGB_STAGE_MOTION: motion_step(w, dt); return 0;
        case AGB_STAGE_SLOW_FIELDS: return slow_fields(w, dt);
        case AGB_STAGE_LIFECYCLE: lifecycle_step(w, dt); return 0;
        case AGB_STAGE_COMPACT: return compact(w);
        case AGB_STAGE_CLOCK: ++w->tick; w->sim_time += dt; return 0;
        case AGB_STAGE_FLASH: flash_step(w, dt); return 0;
        case AGB_STAGE_PREDATION: predation_step(w, dt); return 0;
    }
    return AGB_INVALID_ARGUMENT;
}

int orc_world_step(orc_world* w, int32_t ticks) {
    for (int32_t t = 0; t < ticks; ++t) {
        const double dt = AGB_DT_PHYSICS * w->physics_rate;
        int rc = hash_build(w);
        if (!rc && w->d.thermal_enabled) rc = thermal_step(w, dt);
        if (rc) return rc;
        if (w->d.emission_enabled) emission_step(w, dt);
        if (w->flash_active) flash_step(w, dt);                          /* step.cu:158-162 */
        else if (w->d.taxis_enabled) taxis_step(w, dt);
        motion_step(w, dt);
        rc = slow_fields(w, dt);
        if (rc) return rc;
        predation_step(w, dt);                                            /* step.cu:173-176 */
        lifecycle_step(w, dt);
        ++w->tick;
        w->sim_time += dt;
    }
    return 0;
}

int orc_world_diffuse(orc_world* w, int32_t f, double dt) {
    if (f < 0 || f >= AGB_FIELD_COUNT) return AGB_INVALID_ARGUMENT;
    return grid_diffuse(&w->g[f], dt);
}

int orc_world_counters(orc_world* w, int64_t out[4]) {
    out[0] = w->divisions_this_window;
    out[1] = w->deaths_total;
    out[2] = w->dead_slots_prev;
    out[3] = 0;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Telemetry: src/sim/stats.cu:27-153                                         */
/* ------------------------------------------------------------------------- */
int orc_world_stats(orc_world* w, agb_stats* s) {
    uint64_t energy = 0, temp_cell = 0, temp_medium = 0, co2 = 0, n2 = 0, max_temp = 0;
    uint32_t n_alive = 0, n_dead = 0, n_awake = 0, n_dormant = 0;
    const soa* v = &w->c;
    for (int32_t i = 0; i < w->count; ++i) {               /* stats_cells_kernel, :27-43 */
        const uint32_t f = v->flags[i];
        if (!(f & AGB_FLAG_OCCUPIED)) continue;
        const int alive = (f & AGB_FLAG_ALIVE) != 0u, awake = (f & AGB_FLAG_AWAKE) != 0u;
        if (alive) ++n_alive; else ++n_dead;
        if (awake) ++n_awake; else ++n_dormant;
        energy += (uint64_t)to_fixed(v->energy[i], AGB_DEPOSIT_SCALE_STATS);
        if (alive) temp_cell += (uint64_t)to_fixed((double)v->temp_cell[i], AGB_DEPOSIT_SCALE_STATS);
    }
    const grid *T = &w->g[AGB_FIELD_TEMPERATURE], *C = &w->g[AGB_FIELD_CO2], *N = &w->g[AGB_FIELD_N2];
    if (T->enabled)                                        /* stats_field_kernel, :45-60 */
        for (int64_t i = 0; i < T->count; ++i) {
            const double t = (double)T->value[i];
            temp_medium += (uint64_t)to_fixed(t, AGB_DEPOSIT_SCALE_STATS);
            const uint64_t m = (uint64_t)to_fixed(t, AGB_DEPOSIT_SCALE_STATS);
            if (m > max_temp) max_temp = m;
        }
    if (C->enabled)
        for (int64_t i = 0; i < C->count; ++i) co2 += (uint64_t)to_fixed((double)C->value[i], AGB_STATS_SCALE_FIELD);
    if (N->enabled)
        for (int64_t i = 0; i < N->count; ++i) n2 += (uint64_t)to_fixed((double)N->value[i], AGB_STATS_SCALE_FIELD);
    uint64_t tau_tol = 0;
    uint32_t n_tau = 0;
    for (int32_t i = 0; i < w->tau_count; ++i) {           /* stats_taumoeba_kernel, :65-73 */
        const uint32_t f = w->t.flags[i];
        if (!(f & AGB_FLAG_OCCUPIED) || !(f & AGB_FLAG_ALIVE)) continue;
        ++n_tau;
        tau_tol += (uint64_t)to_fixed((double)w->t.tolerance[i], AGB_DEPOSIT_SCALE_STATS);
    }
    const uint64_t acc[12] = {energy, temp_cell, temp_medium, co2, n2, max_temp, tau_tol,
                              n_alive, n_dead, n_awake, n_dormant, n_tau};
    memcpy(w->accum, acc, sizeof(acc));
    memset(s, 0, sizeof(*s));                              /* world_stats, :102-153 */
    s->tick = w->tick;
    s->sim_time_s = w->sim_time;
    s->physics_rate = w->physics_rate;
    s->biology_rate = w->biology_rate;
    s->n_live = (int32_t)n_alive;
    s->n_dead = (int32_t)n_dead;
    s->n_awake = (int32_t)n_awake;
    s->n_dormant = (int32_t)n_dormant;
    s->n_taumoeba = (int32_t)n_tau;
    s->mean_tau_tolerance = n_tau > 0u ? from_fixed(tau_tol, AGB_DEPOSIT_SCALE_STATS) / n_tau : 0.0;
    s->total_energy_j = from_fixed(energy, AGB_DEPOSIT_SCALE_STATS);
    s->mean_charge = (n_alive + n_dead) > 0u
        ? s->total_energy_j / ((n_alive + n_dead) * AGB_CELL_ENERGY_MAX) : 0.0;
    s->mean_temp_cell_k = n_alive > 0u ? from_fixed(temp_cell, AGB_DEPOSIT_SCALE_STATS) / n_alive : 0.0;
    const double cells = T->enabled ? (double)T->count : 0.0;
    s->mean_temp_medium_k = cells > 0.0 ? from_fixed(temp_medium, AGB_DEPOSIT_SCALE_STATS) / cells : 0.0;
    s->max_temp_medium_k = from_fixed(max_temp, AGB_DEPOSIT_SCALE_STATS);
    const double vc = C->enabled ? C->dx * C->dx * C->dz_eff : 0.0;
    const double vn = N->enabled ? N->dx * N->dx * N->dz_eff : 0.0;
    s->co2_total_kg = from_fixed(co2, AGB_STATS_SCALE_FIELD) * vc;
    s->n2_total_kg = from_fixed(n2, AGB_STATS_SCALE_FIELD) * vn;
    s->divisions_this_window = w->divisions_this_window;
    s->deaths_this_window = (int32_t)(w->deaths_total - w->deaths_reported);
    w->divisions_this_window = 0;
    w->deaths_reported = w->deaths_total;
    s->boil_events = s->max_temp_medium_k >= AGB_WATER_BOILING_POINT ? 1 : 0;
    s->ignitions_this_window = 0;
    s->non_canon_run = 0;
    return 0;
}

int orc_world_stats_accum(orc_world* w, uint64_t out[12]) {
    memcpy(out, w->accum, sizeof(w->accum));
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Snapshot (contracts/snapshot_v1.h:17-63; src/sim/snapshot.cu:100-165)      */
/* ------------------------------------------------------------------------- */
uint64_t orc_fnv1a64(const void* data, uint64_t n, uint64_t h) {
    const unsigned char* p = (const unsigned char*)data;
    for (uint64_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

/* snapshot_to_bytes: header + [overrides][25 cell arrays][20 predator arrays][T, CO2, N2].
 * Returns the byte count; writes into out when cap suffices. */
int64_t orc_world_snapshot(orc_world* w, const char* scenario_id, char* out, int64_t cap) {
    const int stored[3] = {AGB_FIELD_TEMPERATURE, AGB_FIELD_CO2, AGB_FIELD_N2};
    size_t sz[25]; void* p[25];
    soa_sizes(sz); soa_ptrs(&w->c, p);
    const double pmax = w->d.max_emit_power > 0.0 ? w->d.max_emit_power : AGB_PETROVA_MAX_POWER;
    /* OVERRIDE_FIELDS order, snapshot.cu:79-83: emission cap, flash power, division quota. */
    const char* const keys[3] = {"PETROVA_MAX_POWER", "PETROVA_FLASH_POWER", "CO2_MASS_PER_DIVISION"};
    const double vals[3] = {pmax, w->flash_power, w->d.co2_mass_per_division};
    const int on[3] = {pmax != AGB_PETROVA_MAX_POWER, w->flash_power != AGB_PETROVA_FLASH_POWER,
                       w->d.co2_mass_per_division != AGB_CO2_MASS_PER_DIVISION};
    const int has_override = on[0] + on[1] + on[2];
    int64_t body = (int64_t)has_override * (int64_t)sizeof(agb_param_override);
    for (int k = 0; k < 25; ++k) body += (int64_t)sz[k] * w->count;
    for (int k = 0; k < 20; ++k) body += (int64_t)TAU_SZ[k] * w->tau_count;
    for (int k = 0; k < 3; ++k)
        if (w->g[stored[k]].enabled) body += 4 * (int64_t)w->g[stored[k]].count;
    const int64_t total = (int64_t)sizeof(agb_snapshot_header) + body;
    if (!out || cap < total) return total;
    char* q = out + sizeof(agb_snapshot_header);
    for (int o = 0; o < 3; ++o) {
        if (!on[o]) continue;
        agb_param_override ov;
        memset(&ov, 0, sizeof(ov));
        strncpy(ov.key, keys[o], sizeof(ov.key) - 1);
        ov.value = vals[o];
        memcpy(q, &ov, sizeof(ov));
        q += sizeof(ov);
    }
    for (int k = 0; k < 25; ++k) {
        const size_t b = sz[k] * (size_t)w->count;
        if (b) memcpy(q, *(void**)p[k], b);
        q += b;
    }
    {
        void** tp[20];
        tau_ptrs(&w->t, tp);
        for (int k = 0; k < 20; ++k) {
            const size_t b = TAU_SZ[k] * (size_t)w->tau_count;
            if (b) memcpy(q, *tp[k], b);
            q += b;
        }
    }
    for (int k = 0; k < 3; ++k) {
        const grid* g = &w->g[stored[k]];
        if (!g->enabled) continue;
        memcpy(q, g->value, 4 * (size_t)g->count);
        q += 4 * (size_t)g->count;
    }
    agb_snapshot_header h;
    memset(&h, 0, sizeof(h));
    h.magic = AGB_SNAPSHOT_MAGIC;
    h.version = AGB_SNAPSHOT_VERSION;
    h.seed = w->d.seed;
    h.tick = w->tick;
    h.sim_time_s = w->sim_time;
    h.cell_count = w->count;
    h.cell_capacity = w->capacity;
    h.taumoeba_count = w->tau_count;
    h.taumoeba_capacity = w->tau_capacity;
    h.n_temp = w->g[AGB_FIELD_TEMPERATURE].enabled ? w->g[AGB_FIELD_TEMPERATURE].nx : 0;
    h.n_co2 = w->g[AGB_FIELD_CO2].enabled ? w->g[AGB_FIELD_CO2].nx : 0;
    h.n_n2 = w->g[AGB_FIELD_N2].enabled ? w->g[AGB_FIELD_N2].nx : 0;
    h.chamber_w = w->d.chamber_w; h.chamber_h = w->d.chamber_h; h.chamber_d = w->d.chamber_d;
    h.physics_rate = w->physics_rate;
    h.biology_rate = w->biology_rate;
    h.next_cell_id = w->next_id;
    h.override_count = has_override;
    h.non_canon_run = (uint8_t)(has_override > 0);
    if (scenario_id) strncpy(h.scenario_id, scenario_id, sizeof(h.scenario_id) - 1);
    strncpy(h.build_describe, "dev", sizeof(h.build_describe) - 1);
    h.state_hash = orc_fnv1a64(out + sizeof(h), (uint64_t)body, AGB_FNV1A64_OFFSET);
    memcpy(out, &h, sizeof(h));
    return total;
}
