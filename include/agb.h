/*
 * include/agb.h -- C ABI of the GB300 per-tick physics engine (libagb.so).
 *
 * The engine is a drop-in for the simulator's src/sim + src/fields hot path:
 * the spatial hash, thermal coupling + FTCS conduction, the shadowing sweep and
 * feeding, contact forces + the exact Ornstein-Uhlenbeck integrator, CO2 uptake,
 * death, division and stable compaction, and the fixed-point telemetry
 * reduction. Plain C types only; every entry point returns an agb_status.
 *
 * Conventions
 *   - Host buffers are caller-owned; device buffers are engine-owned and are
 *     allocated once at agb_world_create (zero steady-state allocation, the
 *     reference's T29 rule, tests/physics/test_perf.cu:28-74).
 *   - All work is enqueued on the caller's stream; only the explicit export,
 *     stats and count calls synchronise with the host. agb_world_step() never
 *     waits on the device (the reference waits 2-3 times per tick,
 *     src/sim/lifecycle.cu:250-252 and src/sim/cell_store.cu:428).
 *   - One world handle per host thread.
 *   - Status codes 0..9 are astro::Status (src/core/result.h:12-24) one-for-one.
 */
#ifndef AGB_H
#define AGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AGB_ABI_VERSION 1u

typedef int32_t agb_status;
enum {
    AGB_OK = 0,
    AGB_OUT_OF_MEMORY = 1,
    AGB_CUDA_ERROR = 2,
    AGB_INVALID_ARGUMENT = 3,
    AGB_NOT_FOUND = 4,
    AGB_PARSE_ERROR = 5,
    AGB_CONTRACT_VERSION_MISMATCH = 6,
    AGB_CAPACITY_EXCEEDED = 7,
    AGB_FILE_IO_ERROR = 8,
    AGB_UNSUPPORTED = 9,
    /* Not in astro::Status: a bounded device-side wait gave up. */
    AGB_DEVICE_TIMEOUT = 10
};

/* Same object as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* agb_stream;

typedef struct agb_world agb_world;

/* contracts/fields_v1.h:23-27 */
enum { AGB_BC_DIRICHLET = 0, AGB_BC_NEUMANN = 1, AGB_BC_ROBIN = 2 };
/* contracts/fields_v1.h:15-21 */
enum { AGB_FIELD_TEMPERATURE = 0, AGB_FIELD_CO2 = 1, AGB_FIELD_N2 = 2, AGB_FIELD_IRRADIANCE = 3,
       AGB_FIELD_COUNT = 4 };
/* src/sim/integrator.cuh:227 Boundary, :175 GravityAxis */
enum { AGB_WALL_REFLECTING = 0, AGB_WALL_PERIODIC = 1, AGB_WALL_ABSORBING = 2 };
enum { AGB_GRAVITY_Y = 0, AGB_GRAVITY_Z = 1 };
/* contracts/scenario_v3.h:35 StoreDisposition */
enum { AGB_STORE_VOID = 0, AGB_STORE_FLASH = 1, AGB_STORE_RETAIN = 2 };
/* Division predicate. CO2 quota is the reference (src/sim/lifecycle.cuh:33-36);
 * the stored-energy threshold is an opt-in extension, not reference behaviour. */
enum { AGB_DIVIDE_CO2_QUOTA = 0, AGB_DIVIDE_ENERGY = 1 };
/* src/sim/world.cuh:33 BrushKind */
enum { AGB_BRUSH_HEAT = 0, AGB_BRUSH_CHILL = 1, AGB_BRUSH_INJECT_CO2 = 2, AGB_BRUSH_INJECT_N2 = 3 };
/* Face order of agb_grid_desc.bc / face_value. */
enum { AGB_FACE_XMIN = 0, AGB_FACE_XMAX = 1, AGB_FACE_YMIN = 2, AGB_FACE_YMAX = 3,
       AGB_FACE_ZMIN = 4, AGB_FACE_ZMAX = 5 };

/*
 * One scalar field on a regular grid (src/fields/grid.cuh:72-85 Grid2D,
 * contracts/fields_v1.h:81-91 FieldView). The x spacing is dx = chamber_w / nx
 * and y uses the same dx, as in the reference. nz == 1 is the reference's
 * depth-averaged 2-D grid, bit for bit; nz > 1 is a 3-D grid with
 * dz = chamber_d / nz, which must equal dx (isotropic 7-point stencil).
 * nx == 0 disables the field (it is then never sampled, diffused or stored).
 */
typedef struct agb_grid_desc {
    int32_t nx, ny, nz;
    int32_t bc[6];            /* per face, AGB_FACE_* order; the reference uses one bc for all */
    double face_value[6];     /* Dirichlet value / Robin reference temperature per face */
    double diffusivity;       /* [m^2/s] */
    double init;              /* uniform initial value (the reference fills with its ambient) */
    double deposit_scale;     /* fixed-point scale of the deposit accumulator */
} agb_grid_desc;

/* contracts/fields_v1.h:106-111 LightSource + World::ambient_irradiance.
 * The sweep runs along the dominant axis of dir (ties: x, then y, then z);
 * the reference only has in-plane x/y light (src/sim/emission.cu:161-163). */
typedef struct agb_light {
    float dir_x, dir_y, dir_z;
    float irradiance;         /* [W/m^2] at the illuminated boundary */
    float ambient;            /* [W/m^2] isotropic ambient */
    int32_t enabled;
} agb_light;

/* WorldDesc + MotionConfig + the World knobs the tick reads
 * (src/sim/world.cuh:48-180). agb_world_desc_default() fills the reference's
 * defaults (src/sim/step.cu:9-78, src/sim/world.cuh:48-87). */
typedef struct agb_world_desc {
    uint32_t abi_version;     /* AGB_ABI_VERSION */
    double chamber_w, chamber_h, chamber_d;   /* [m], centred on the origin */
    int32_t capacity;         /* cell slots */
    uint64_t seed;
    int32_t boundary_x, boundary_y, gravity_axis;
    uint8_t thermal_noise, contact_enabled, adhesion_enabled, thermal_enabled;
    uint8_t emission_enabled, taxis_enabled, occlusion_exact, compaction_enabled;
    int32_t store_disposition;
    double ambient_temp;      /* [K] */
    agb_grid_desc grid[AGB_FIELD_COUNT];
    double hash_cell_size;    /* [m]; the reference uses HASH_CELL_FACTOR * CELL_DIAMETER */
    agb_light light;
    double physics_rate, biology_rate;
    double co2_mass_per_division;             /* [kg] World override, canon by default */
    double max_emit_power;                    /* [W] World::petrova_max_power, canon by default */
    /* Extensions; the defaults reproduce the reference. */
    int32_t division_predicate;               /* AGB_DIVIDE_* */
    double division_energy;                   /* [J] threshold for AGB_DIVIDE_ENERGY */
    int32_t compaction_period;                /* ticks between compaction checks; 1 = reference */
    int32_t trap_slot;                        /* optical trap (World::trap_*); -1 = off */
    double trap_x, trap_y, trap_stiffness;
    /* The predator store (WorldDesc::tau_capacity, MotionConfig::tau_compaction_enabled,
     * src/sim/world.cuh:76-82): capacity, 0 = AGB_DEFAULT_TAUMOEBA; stable compaction of
     * dead predators. */
    int32_t tau_capacity;
    int32_t tau_compaction_enabled;
} agb_world_desc;

/* CellStoreView (contracts/cell_store_v1.h:42-78), member for member and at the
 * same offsets: the 25 SoA arrays, then count and capacity, so a reference
 * caller's view can be passed as it is. Any pointer may be NULL in export
 * calls (that array is skipped). The import calls take the cell count as an
 * argument and ignore `count` and `capacity` here; the export calls set
 * `count` to the population and `capacity` to the caller's array length;
 * agb_world_device_cells sets both from the store. */
typedef struct agb_cells {
    uint64_t* id;
    uint32_t* flags;
    uint8_t* death_cause;
    double *x, *y, *z;
    double *vx, *vy, *vz;
    double* energy;
    float* temp_cell;
    float* emit_power;
    float *dir_x, *dir_y, *dir_z;
    double* biomass;
    double* co2_held;
    float* age_s;
    uint64_t* rng_state;
    float* taxis_memory;
    float* run_timer;
    float* t_local;
    float* irradiance;
    float* co2_local;
    float* n2_local;
    int32_t count;
    int32_t capacity;
} agb_cells;

/* src/sim/cell_store.cuh:15-28 SpawnParams. Placements 0-3 and distributions
 * 0-2 are the reference's (src/sim/cell_store.cu:42-130); the rest generate the
 * benchmark workloads and are extensions:
 *   AGB_PLACE_SLAB_X   x uniform in place_x +- place_radius, y over the chamber,
 *                      z as the reference (uniform through the depth);
 *   AGB_PLACE_CLUSTERS a 3-D Gaussian mixture: `clusters` centres uniform in a
 *                      cube of edge cluster_extent, sigma = place_radius;
 *   AGB_DIST_LOGNORMAL charge = exp(ln(charge_a) + charge_b * N(0,1)).
 * charge_max > 0 clips the charge from above after the reference's clamp to [0,1]. */
enum { AGB_PLACE_UNIFORM = 0, AGB_PLACE_GAUSSIAN = 1, AGB_PLACE_GRID = 2, AGB_PLACE_DISC = 3,
       AGB_PLACE_SLAB_X = 4, AGB_PLACE_CLUSTERS = 5 };
enum { AGB_DIST_CONSTANT = 0, AGB_DIST_UNIFORM = 1, AGB_DIST_NORMAL = 2, AGB_DIST_LOGNORMAL = 3 };
typedef struct agb_spawn {
    int32_t count, placement, charge_dist, awake;
    double place_x, place_y, place_radius;
    double charge_a, charge_b;
    double charge_max;
    int32_t clusters;
    double cluster_extent;
} agb_spawn;

/* contracts/telemetry_v1.h:17-39 Stats, same members in the same order. */
typedef struct agb_stats {
    uint64_t tick;
    double sim_time_s;
    int32_t n_live, n_dead, n_dormant, n_awake, n_taumoeba;
    double mean_charge;
    double total_energy_j;
    double mean_temp_cell_k;
    double mean_temp_medium_k;
    double max_temp_medium_k;
    double co2_total_kg;
    double n2_total_kg;
    double mean_tau_tolerance;
    int32_t divisions_this_window;
    int32_t deaths_this_window;
    int32_t boil_events;
    int32_t ignitions_this_window;
    double physics_rate, biology_rate;
    uint8_t non_canon_run;
} agb_stats;

/* Stages of world_step (src/sim/step.cu:109-184), for stage-level parity. */
enum {
    AGB_STAGE_HASH = 0,        /* hash_build, src/sim/hash.cu:106-133 */
    AGB_STAGE_THERMAL = 1,     /* thermal_step, src/sim/thermal.cu:75-103 */
    AGB_STAGE_EMISSION = 2,    /* emission_step, src/sim/emission.cu:119-177 */
    AGB_STAGE_TAXIS = 3,       /* taxis_step, src/sim/taxis.cu:80-85 */
    AGB_STAGE_MOTION = 4,      /* motion_step, src/sim/integrator.cu:154-177 */
    AGB_STAGE_SLOW_FIELDS = 5, /* CO2/N2 flush + diffuse, src/sim/step.cu:168-171 */
    AGB_STAGE_LIFECYCLE = 6,   /* lifecycle_step, src/sim/lifecycle.cu:208-294 */
    AGB_STAGE_COMPACT = 7,     /* cell_store_compact, src/sim/cell_store.cu:414-456 */
    AGB_STAGE_CLOCK = 8,       /* ++tick; sim_time += dt, src/sim/step.cu:182-183 */
    AGB_STAGE_FLASH = 9,       /* flash_step, src/sim/flash.cu:59-67 (a no-op unless armed) */
    AGB_STAGE_PREDATION = 10   /* predation_step, src/sim/predation.cu:434-484 */
};

/* Snapshots (contracts/snapshot_v1.h:17-63): file = header, then the body the
 * state hash covers: overrides, the 25 cell arrays (contract order, count
 * elements each), predator arrays (none in this engine), T, CO2, N2 values.
 * Little-endian; the layout below is the contract's, field for field. */
#define AGB_SNAPSHOT_MAGIC 0x48505341u          /* 'ASPH' */
#define AGB_SNAPSHOT_VERSION 1u
#define AGB_FNV1A64_OFFSET 1469598103934665603ull

typedef struct agb_snapshot_header {
    uint32_t magic, version;
    uint64_t seed, tick;
    double sim_time_s;
    int32_t cell_count, cell_capacity;
    int32_t taumoeba_count, taumoeba_capacity;
    int32_t n_temp, n_co2, n_n2;                /* grid nx (the reference's n of an n x n grid) */
    int32_t _pad0;                              /* natural alignment of the double that follows */
    double chamber_w, chamber_h, chamber_d;
    double physics_rate, biology_rate;
    uint64_t next_cell_id;
    int32_t override_count;
    uint8_t non_canon_run;
    uint8_t _pad[3];
    char scenario_id[64];
    char build_describe[64];
    uint64_t state_hash;                        /* FNV-1a 64 over the body */
} agb_snapshot_header;

typedef struct agb_param_override {
    char key[48];
    double value;
} agb_param_override;

/* The learned field surrogate (no counterpart in the reference): advances the
 * temperature and CO2 grids `steps` FTCS steps per call with a 3-level 3-D
 * convolutional encoder-decoder (32/64/128 channels, 3x3x3 kernels, BF16
 * weights and activations, FP32 accumulation, tensor cores), trained on the
 * GPU on seeded FTCS windows. Every judge_every-th call also runs the plain
 * FTCS window and falls back to its result when the largest temperature
 * error exceeds tol_temperature or the relative drift of the summed
 * temperature exceeds tol_energy. The window operator on both fields is
 * `steps` times X <- FTCS(X + q) with constant per-step sources q. */
typedef struct agb_surrogate agb_surrogate;

typedef struct agb_surrogate_desc {
    uint32_t abi_version;
    int32_t nx, ny, nz;               /* nx 128 or 256; ny a multiple of 16; nz a multiple of 4 */
    double extent;                    /* chamber width (m): dx = extent / nx, cubic voxels */
    double dt;                        /* seconds per FTCS step */
    int32_t steps;                    /* FTCS steps per call (16) */
    int32_t judge_every;              /* judge every k-th call (8) */
    double tol_temperature;           /* K (0.01) */
    double tol_energy;                /* relative (1e-6) */
    double diffusivity[2];            /* temperature, CO2 (m^2/s) */
    double init[2];                   /* reference values the inputs are normalised about */
    int32_t bc[2][6];                 /* boundary conditions per field and face */
    double face[2][6];
    uint64_t seed;
    float learning_rate;
    double train_temperature_amplitude;   /* K: blob amplitude of the training windows */
    double train_source_density;          /* fraction of voxels holding a source */
    double train_heat_per_step;           /* K per step: largest heating source */
    double train_uptake_per_step;         /* kg/m^3 per step: largest CO2 uptake */
} agb_surrogate_desc;

typedef struct agb_surrogate_report {
    int64_t calls, judged, fallbacks;
    double last_err_temperature;      /* K, last judged call */
    double last_err_co2;
    double last_energy_drift;
    int32_t last_used_surrogate;      /* 0: the last call's output is the judge's FTCS result */
    float last_loss;                  /* last training loss (mean squared normalised error) */
} agb_surrogate_report;

/* Batched ensembles (no counterpart in the reference, which runs one World per
 * process): N independent chambers of uneven cell counts and grid sizes, each
 * a full world, advanced together by one CUDA graph launch per
 * agb_batch_step call. */
typedef struct agb_batch agb_batch;
#define AGB_BATCH_MAX_CHAMBERS 4096

typedef struct agb_batch_opts {
    uint32_t abi_version;       /* AGB_ABI_VERSION */
    int32_t lanes;              /* concurrent branches of the batch graph; 0 = min(n, 16) */
    int32_t autotune;           /* 1: time candidate hash cells and stencil tilings per size class */
    int32_t n_hash_candidates;  /* 0: 1.0, 1.5, 2.2 and 3.0 cell diameters */
    double hash_candidates[8];  /* metres; candidates under one cell diameter are skipped */
    int32_t probe_ticks;        /* timed probe ticks per candidate (0 = 4) */
    int32_t staged;             /* 1 (default): each stage of the tick is one launch over every chamber,
                                   when every enabled grid is 3-D with a TMA stencil, no chamber has a
                                   surrogate attached and none exceeds ~67M cells of capacity; 0: each
                                   chamber's tick is launched on the lanes */
} agb_batch_opts;

/* What a chamber was built with, and what the autotuner measured for it. */
typedef struct agb_tuning {
    double hash_cell_size;      /* metres */
    int32_t size_class;         /* chambers sharing temperature grid edge and cell-count decade */
    int32_t lane;               /* branch of the batch graph */
    int32_t ftcs_lx[3], ftcs_rpt[3], ftcs_zc[3];   /* stencil tiling of T, CO2, N2 (0: no TMA path) */
    float probe_tick_ms;        /* best probe tick of the class (0 when not tuned) */
    float probe_pass_us;        /* best probe FTCS pass of the class's temperature grid */
} agb_tuning;

/* Reference defaults: 4 mm x 4 mm x 60 um slab, 512^2 temperature (Robin),
 * 256^2 CO2, 128^2 N2 and 512^2 irradiance grids (all nz = 1), canon hash. */
void agb_world_desc_default(agb_world_desc* d);

const char* agb_status_str(agb_status s);
const char* agb_last_error(const agb_world* w);
/* CUDA device the engine runs on and its compute capability (e.g. 103). */
agb_status agb_device_info(int32_t* device, int32_t* sm_version, int32_t* sm_count);

/* world_create / world_destroy (src/sim/world.cuh:222-223). */
agb_status agb_world_create(const agb_world_desc* d, agb_world** out);
void agb_world_destroy(agb_world* w);

/* cell_store_spawn (src/sim/cell_store.cuh:73): appends p->count seeded cells. */
agb_status agb_world_spawn(agb_world* w, const agb_spawn* p, agb_stream s);
/* The same with the spawn seed given (cell_store_spawn's `seed` argument; the call
 * above passes the world's seed): the scenario loader seeds population i with
 * seed + i and a top-up with seed + tick (src/sim/scenario.cpp:368-385, 436-452). */
agb_status agb_world_spawn_seeded(agb_world* w, const agb_spawn* p, uint64_t seed, agb_stream s);

/* cell_store_set_charge (src/sim/cell_store.cuh:78): every occupied slot's
 * stored energy set to clamp(charge, 0, 1) * CELL_ENERGY_MAX. */
agb_status agb_world_set_charge(agb_world* w, double charge, agb_stream s);

/* Replace the whole population with `count` cells in contract layout; next_id
 * is the id the next daughter gets (CellStore::next_id). */
agb_status agb_world_import_cells(agb_world* w, const agb_cells* src, int32_t count,
                                  uint64_t next_id, agb_stream s);
/* Copy up to max_count cells out; writes the live upper bound and next_id. Syncs. */
agb_status agb_world_export_cells(agb_world* w, agb_cells* dst, int32_t max_count,
                                  int32_t* count, uint64_t* next_id, agb_stream s);
/* Device pointers of the SoA (the reference's CellStore::view); count via agb_world_count. */
agb_status agb_world_device_cells(agb_world* w, agb_cells* dev);

/* Host view of the predator store's 20 arrays (TaumoebaStore, src/sim/predation.cuh:85-105),
 * field for field, in the snapshot's order. Any pointer may be NULL on export. */
typedef struct agb_taumoeba {
    uint64_t* id;
    uint32_t* flags;
    double *x, *y, *z;
    double *vx, *vy, *vz;
    float *dir_x, *dir_y, *dir_z;
    double* biomass;
    double* prey_biomass;
    float* digest_timer;
    float* tolerance;
    uint32_t* generation;
    uint64_t* rng_state;
    float* density_ema;
    float* run_timer;
    int32_t* target;
} agb_taumoeba;
/* taumoeba_spawn (src/sim/predation.cu:420-432): append `count` predators placed uniformly,
 * streams seeded from (splitmix64(seed), id). Capacity exceeded is an error. */
agb_status agb_world_spawn_taumoeba(agb_world* w, int32_t count, uint64_t seed, agb_stream s);
/* Replace the predator store with `count` predators; next_id is the next predator id. */
agb_status agb_world_import_taumoeba(agb_world* w, const agb_taumoeba* src, int32_t count, uint64_t next_id,
                                     agb_stream s);
/* Copy up to max_count predators out (the taumoeba_download_* readers). Syncs. */
agb_status agb_world_export_taumoeba(agb_world* w, agb_taumoeba* dst, int32_t max_count, int32_t* count,
                                     uint64_t* next_id, agb_stream s);
/* One call per host-driven step: import `count` cells from host arrays, run
 * `ticks` ticks (one graph launch), export into host arrays (at most max_out
 * per array) and synchronise once. With device-accessible host arrays
 * (pinned, or host page tables) both transfers are single kernels over the
 * host link. */
agb_status agb_world_step_host(agb_world* w, const agb_cells* in, int32_t count, uint64_t next_id,
                               int32_t ticks, agb_cells* out, int32_t max_out, int32_t* out_count,
                               uint64_t* out_next_id, agb_stream s);
agb_status agb_world_count(agb_world* w, int32_t* count, agb_stream s);

/* Field values, nx*ny*nz floats, x fastest (reference: [x + n*y]). */
agb_status agb_world_import_field(agb_world* w, int32_t field, const float* src, agb_stream s);
agb_status agb_world_export_field(agb_world* w, int32_t field, float* dst, agb_stream s);
/* Raw fixed-point accumulator (irradiance: the occlusion stamp of the last emission stage). */
agb_status agb_world_export_deposit(agb_world* w, int32_t field, uint64_t* dst, agb_stream s);

/* The spin-drive flash (World::flash_active / petrova_flash_power, src/sim/world.cuh:169-179):
 * while armed, each tick's flash stage replaces taxis (src/sim/step.cu:158-162) and every
 * awake charged cell discharges power * dt of its store (src/sim/flash.cu:31-56); power <= 0
 * takes the canon AGB_PETROVA_FLASH_POWER. Call between ticks. */
agb_status agb_world_set_flash(agb_world* w, int32_t active, double power);
/* world_flash_audit (src/sim/flash.cu:69-78): delivered impulse [N s] and discharged store [J]
 * since creation. Synchronises. */
agb_status agb_world_flash_audit(agb_world* w, double* impulse_ns, double* discharged_j);

/* world_apply_brush (src/sim/step.cu:80-89, grid_brush src/fields/diffuse.cu:81-89): add
 * strength * (1 - (r/radius)^2)^2 to the kind's field (chill: subtract) at voxels whose
 * centre lies within `radius` [m] of (x, y) in the chamber frame; a 3-D grid takes the disc on
 * every z plane. radius <= 0 is a no-op. Call between ticks; no host synchronisation.
 * Errors: unknown kind, non-finite arguments, or a field the world does not have. */
agb_status agb_world_apply_brush(agb_world* w, int32_t kind, double x, double y, double radius,
                                 double strength, agb_stream s);

/* world_step x ticks (src/sim/step.cu:109-184). No host synchronisation. */
agb_status agb_world_step(agb_world* w, int32_t ticks, agb_stream s);
/* Capture `ticks` ticks once as a CUDA graph and replay it on later calls with
 * the same tick count: one launch per call. */
agb_status agb_world_step_graph(agb_world* w, int32_t ticks, agb_stream s);
/* Captures, without running them, the graphs agb_world_step_graph(w, ticks, .)
 * will replay from the world's current state on: one per (field buffer
 * parities, tick % compaction_period) state that stepping by `ticks` visits,
 * until the states repeat. Afterwards no step of that size captures or
 * instantiates anything (no host-side latency spike in a serving loop or a
 * timed region). The world's state is unchanged. No counterpart in the
 * reference (its world_step has no graphs). */
agb_status agb_world_prepare_graphs(agb_world* w, int32_t ticks, agb_stream s);
/* Section timers: with timing on, every tick (eager or captured into a graph)
 * records a pair of timing events around each section below, so the times of
 * the kernels inside a replayed graph can be read without a profiler. The
 * event nodes end the programmatic (early) launch of the kernel after them, so
 * timed ticks run slightly slower; off by default. Switching invalidates the
 * world's captured graphs. agb_world_section_times waits for the last tick and
 * returns each section's duration in milliseconds (-1 for a section that has
 * not run). No counterpart in the reference. */
enum {
    AGB_SECTION_TICK = 0,        /* the whole tick, first launch to last */
    AGB_SECTION_THERMAL = 1,     /* thermal substeps (all but the last pass's flush and FTCS) */
    AGB_SECTION_T_DIFFUSE = 2,   /* last temperature flush + FTCS pass */
    AGB_SECTION_IRRADIANCE = 3,  /* stamps, occlusion factors, sweep */
    AGB_SECTION_SLOW_FIELDS = 4, /* CO2 / N2 FTCS passes */
    AGB_SECTION_HASH = 5,        /* keys, radix sort, bucket ranges */
    AGB_SECTION_CELL_PASS = 6,   /* feeding, taxis and forces (fused or separate) */
    AGB_SECTION_INTEGRATE = 7,   /* OU integration (+ CO2 demand) */
    AGB_SECTION_LIFECYCLE = 8,   /* predation, uptake, death, division, compaction */
    AGB_TICK_SECTIONS = 9
};
agb_status agb_world_set_timing(agb_world* w, int32_t enable);
agb_status agb_world_section_times(agb_world* w, float ms[AGB_TICK_SECTIONS]);
/* Kernel launches performed by graph replays since the world was created
 * (the sum of each replayed graph's kernel nodes), for launch accounting. */
agb_status agb_world_graph_kernels(agb_world* w, int64_t* kernels);
/* How a tick runs the neighbour walks of feeding (src/sim/emission.cu:81-115)
 * and contact forces (src/sim/integrator.cu:40-76): `lanes` threads share each
 * cell's walk (1, 2, 4 or 8), and `fused` = 1 runs feeding, taxis and forces
 * as one kernel with one walk per cell, 0 as separate kernels. Default: 2
 * lanes fused for capacities up to 512 cells per SM, else 1 lane separate;
 * chambers of a batch use 1 lane. Results agree to FP32
 * summation order; integer state is unchanged. Captured graphs are rebuilt.
 * No reference counterpart (a launch-shape knob of this engine). */
agb_status agb_world_set_walk(agb_world* w, int32_t lanes, int32_t fused);
agb_status agb_world_walk(agb_world* w, int32_t* lanes, int32_t* fused);
/* One stage of the tick at the world's dt (AGB_STAGE_*). */
agb_status agb_world_stage(agb_world* w, int32_t stage, agb_stream s);
/* grid_diffuse on one field for dt (src/fields/diffuse.cu:159-186). */
agb_status agb_world_diffuse(agb_world* w, int32_t field, double dt, agb_stream s);

/* Diffusion of one field the caller owns in device memory, with no device
 * allocation: grid_diffuse's substepping and arithmetic (bit for bit), with the
 * second ping-pong buffer taken from a fixed scratch array inside the library
 * (AGB_NOALLOC_MAX_VOXELS floats, 16 MiB, held on every GPU that loads the
 * library until the process exits). This entry point has no counterpart in
 * the reference. It exists for callers that may not allocate device memory:
 * applications with a fixed device-memory budget reserved at start-up, plugins
 * inside a host that owns the CUDA context's allocation policy, and real-time
 * loops that cannot afford cudaMalloc's implicit synchronisation.
 * `value` is nx*ny*nz floats, x fastest; dx is the isotropic spacing; bc and
 * face_value follow agb_grid_desc; the result is left in `value`.
 * Returns AGB_CAPACITY_EXCEEDED for grids larger than AGB_NOALLOC_MAX_VOXELS,
 * and AGB_UNSUPPORTED for grids within it whose stencil launch would need more
 * than 65,535 blocks along y or z (ny > 524,280, or nz > 524,280); in both
 * cases nothing is launched and `value` is untouched. If a stencil pass fails
 * to launch, the call returns AGB_CUDA_ERROR before its final copy into
 * `value`. The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the scratch array: calls whose work overlaps on the GPU race.
 * Its contents are left over from the previous call and need no clearing. */
#define AGB_NOALLOC_MAX_VOXELS 4194304
agb_status agb_grid_diffuse_noalloc(float* value, int32_t nx, int32_t ny, int32_t nz, double dx,
                                    double diffusivity, double dt, const int32_t bc[6],
                                    const double face_value[6], agb_stream s);

/* world_stats (src/sim/stats.cu:102-153): fixed-point reduction + window counters. Syncs. */
agb_status agb_world_stats(agb_world* w, agb_stats* out, agb_stream s);
/* The raw fixed-point sums of the last agb_world_stats, StatsAccum order
 * (src/sim/world.cuh:39-45): energy, temp_cell, temp_medium, co2, n2, max_temp,
 * tau_tolerance, n_alive, n_dead, n_awake, n_dormant, n_taumoeba. */
agb_status agb_world_stats_accum(agb_world* w, uint64_t out[12]);

/* world_set_clock with explicit rates (src/sim/step.cu:196-205, clamped). */
agb_status agb_world_set_clock(agb_world* w, double physics_rate, double biology_rate);
agb_status agb_world_set_light(agb_world* w, const agb_light* light);
/* The rates as a caller assigns World::physics_rate / biology_rate directly
 * (src/sim/step.cu:133 reads them unclamped): finite and positive. */
agb_status agb_world_set_rates(agb_world* w, double physics_rate, double biology_rate);
/* The live overrides World::co2_mass_per_division and World::petrova_max_power
 * (src/sim/world.cuh:171-173), assigned between ticks. */
agb_status agb_world_set_overrides(agb_world* w, double co2_mass_per_division, double max_emit_power);


/* A field's boundary between ticks (the caller assigning Grid2D::bc,
 * src/fields/grid.cuh:84, as tests/physics/test_thermal.cu does): per face kind
 * (AGB_BC_*) and Dirichlet value / Robin reference, AGB_FACE_* order. */
agb_status agb_world_set_boundary(agb_world* w, int32_t field, const int32_t bc[6], const double face_value[6]);

/* Hash state after the last hash stage: dims = {nx, ny, nz, bucket_count};
 * keys/vals in sorted order (count entries); bucket_start/end dense
 * (bucket_count entries, empty buckets 0/0 as in src/sim/hash.cu:110-113). Syncs. */
agb_status agb_world_export_hash(agb_world* w, int32_t dims[4], uint32_t* keys_sorted,
                                 uint32_t* vals_sorted, int32_t* bucket_start,
                                 int32_t* bucket_end, agb_stream s);
/* Net force per slot of the last motion stage (World::d_fx/fy/fz). Syncs. */
agb_status agb_world_export_forces(agb_world* w, float* fx, float* fy, float* fz, agb_stream s);
/* Device counters: {divisions_this_window, deaths_total, dead_slots_prev,
 * device error word}. Syncs. */
agb_status agb_world_counters(agb_world* w, int64_t out[4], agb_stream s);

/* What a host-side mirror of the world needs after a tick (the reference's
 * World members that callers read between ticks, src/sim/world.cuh:110-128 and
 * cell_store.cuh:36-43), read with one synchronisation: the cell store's device
 * view with count and capacity (as agb_world_device_cells), the next cell id,
 * the lifecycle counters and error word (as agb_world_counters), and the
 * predator count and next id. */
typedef struct agb_mirror {
    agb_cells cells;
    uint64_t next_id;
    int64_t divisions_this_window;
    int64_t deaths_total;
    int64_t dead_slots_prev;
    uint32_t error;
    int32_t tau_count;
    uint64_t tau_next_id;
} agb_mirror;
agb_status agb_world_mirror(agb_world* w, agb_mirror* out, agb_stream s);

/* fnv1a64 (contracts/snapshot_v1.h:57-61): h = (h ^ byte) * 1099511628211,
 * starting from h (AGB_FNV1A64_OFFSET for a fresh hash). */
uint64_t agb_fnv1a64(const void* data, uint64_t n, uint64_t h);
/* snapshot_state_hash (src/sim/snapshot.cu:126-132): FNV-1a of the body. */
agb_status agb_world_state_hash(agb_world* w, uint64_t* hash, agb_stream s);
/* snapshot_to_bytes (src/sim/snapshot.cu:134-165). buf == NULL: only *size is
 * set; a cap under *size returns AGB_CAPACITY_EXCEEDED and writes nothing. */
agb_status agb_world_snapshot_save(agb_world* w, const char* scenario_id, void* buf, int64_t cap,
                                   int64_t* size, agb_stream s);
/* snapshot_from_bytes (src/sim/snapshot.cu:167-246): the motion configuration
 * and grid layout come from *base (the snapshot does not carry them), the
 * chamber, capacity, seed, clock rates and state from the snapshot. A corrupt
 * body (hash mismatch), bad magic or a grid resolution that differs from the
 * header fails as the reference does. */
agb_status agb_world_snapshot_load(const agb_world_desc* base, const void* data, int64_t n, agb_world** out);

/* Learned-surrogate layer primitives on caller-owned device buffers (no
 * counterpart in the reference). Activations are channels-last BF16
 * [D][H][W][C], weights [27][cout][cin] BF16 with tap (dz+1)*9+(dy+1)*3+(dx+1).
 * agb_nn_conv3: 3x3x3 "same" convolution on the tensor cores, out =
 * act(conv(x, w) + bias), zeroed where mask <= 0 when mask is given; BF16 or
 * FP32 output. agb_nn_wgrad: dw[27][cout][cin] (and db[cout] when given) of
 * that convolution from its input x and output gradient dy, FP32, using
 * agb_nn_wgrad_scratch_bytes of scratch. agb_nn_flip_weights: the weights of
 * the input-gradient convolution, wf[26-t][ci][co] = w[t][co][ci]. err is a
 * device word set nonzero when a bounded wait inside a kernel expired. */
agb_status agb_nn_conv3(const void* x, const void* w, const float* bias, int32_t D, int32_t H, int32_t W,
                        int32_t cin, int32_t cout, int32_t act, const void* mask, void* out, int32_t out_f32,
                        uint32_t* err, agb_stream s);
int64_t agb_nn_wgrad_scratch_bytes(int32_t D, int32_t H, int32_t W, int32_t cin, int32_t cout);
agb_status agb_nn_wgrad(const void* x, const void* dy, int32_t D, int32_t H, int32_t W, int32_t cin, int32_t cout,
                        float* dw, float* db, void* scratch, int64_t scratch_bytes, uint32_t* err, agb_stream s);
agb_status agb_nn_flip_weights(const void* w, void* wf, int32_t cout, int32_t cin, agb_stream s);

/* Surrogate lifetime, training and use. Field pointers are device buffers of
 * nx*ny*nz floats. agb_surrogate_train trains on `windows` seeded windows
 * (losses[k] per window when given). agb_surrogate_advance updates T and C in
 * place by one window; judge: 1 forces the judge, -1 skips it, 0 follows
 * judge_every. agb_surrogate_reference is the plain FTCS window (the method
 * without the network); agb_surrogate_window writes training window `index`.
 * agb_surrogate_gradients runs one forward and backward pass against given
 * targets without updating (for gradient checks); parameters and gradients
 * are flat FP32 in layer order, each layer's [27][cout][cin] weights then its
 * cout biases. */
void agb_surrogate_desc_default(agb_surrogate_desc* d);
agb_status agb_surrogate_create(const agb_surrogate_desc* d, agb_surrogate** out);
void agb_surrogate_destroy(agb_surrogate* s);
agb_status agb_surrogate_train(agb_surrogate* s, int32_t windows, float* losses, agb_stream st);
/* One training step on a window the caller supplies (device arrays on the
 * surrogate's grid: temperature, CO2 and the per-step sources, NULL sources
 * = none), e.g. fields and rasterised cell sources taken from world runs; its
 * target is the plain FTCS window from those fields. *loss (optional, host)
 * receives the step's loss (the call then waits for it). */
agb_status agb_surrogate_train_on(agb_surrogate* s, const float* T0, const float* C0, const float* qT,
                                  const float* qC, float* loss, agb_stream st);
agb_status agb_surrogate_advance(agb_surrogate* s, float* T, float* C, const float* qT, const float* qC,
                                 int32_t judge, agb_surrogate_report* rep, agb_stream st);
agb_status agb_surrogate_reference(agb_surrogate* s, float* T, float* C, const float* qT, const float* qC,
                                   agb_stream st);
agb_status agb_surrogate_window(agb_surrogate* s, uint64_t index, float* T, float* C, float* qT, float* qC,
                                agb_stream st);
agb_status agb_surrogate_gradients(agb_surrogate* s, const float* T0, const float* C0, const float* qT,
                                   const float* qC, const float* T1, const float* C1, float* grads, int64_t cap,
                                   float* loss, agb_stream st);
agb_status agb_surrogate_params(agb_surrogate* s, float* out, int64_t cap, int64_t* count);
agb_status agb_surrogate_set_params(agb_surrogate* s, const float* in, int64_t count);
agb_status agb_surrogate_get_report(agb_surrogate* s, agb_surrogate_report* rep);
agb_status agb_surrogate_error_word(agb_surrogate* s, uint32_t* word);
/* Let the surrogate drive a world's temperature and CO2 grids (NULL detaches).
 * The grids, the one-pass-per-tick FTCS coefficients and the boundary
 * conditions must be the surrogate's. While attached, the cells' heat
 * exchange accumulates over each window of `steps` ticks and becomes the
 * window's per-step source; neither grid is diffused tick by tick; at the end
 * of each window the surrogate (and, every judge_every-th window, its FTCS
 * judge) advances both grids. Steps run eagerly (no graph capture). */
agb_status agb_world_attach_surrogate(agb_world* w, agb_surrogate* sg, agb_stream s);

/* Batches. agb_batch_create builds chamber i from descs[i], seeds it with
 * spawns[i] (may be NULL: no cells) and, with opts->autotune, first picks each
 * size class's hash cell size and stencil tilings by timing probe chambers.
 * agb_batch_step advances every chamber by `ticks` ticks in one graph launch
 * on s (NULL: the batch's own stream); each chamber's result equals a
 * standalone world built with agb_batch_tuning's hash cell size. Chamber
 * handles from agb_batch_world are owned by the batch and accept every
 * agb_world_* call between steps. agb_batch_stats fills n agb_stats. */
void agb_batch_opts_default(agb_batch_opts* o);
agb_status agb_batch_create(const agb_world_desc* descs, const agb_spawn* spawns, int32_t n,
                            const agb_batch_opts* opts, agb_batch** out);
void agb_batch_destroy(agb_batch* b);
const char* agb_batch_last_error(const agb_batch* b);
agb_status agb_batch_size(agb_batch* b, int32_t* n);
agb_status agb_batch_world(agb_batch* b, int32_t i, agb_world** w);
agb_status agb_batch_tuning(agb_batch* b, int32_t i, agb_tuning* out);
agb_status agb_batch_step(agb_batch* b, int32_t ticks, agb_stream s);
agb_status agb_batch_graph_kernels(agb_batch* b, int64_t* kernels);
/* 1 when steps run staged (one launch per stage over every chamber), 0 on lanes. */
agb_status agb_batch_staged(agb_batch* b, int32_t* staged);
agb_status agb_batch_stats(agb_batch* b, agb_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* AGB_H */
