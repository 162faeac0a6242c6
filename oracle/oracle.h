/*
 * oracle/oracle.h -- CPU oracle of the per-tick physics step.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use this; the product (libagb.so) never links it. It is a plain-C
 * restatement of the reference's kernel bodies (src/sim/*.cu, src/fields/*.cu)
 * in the reference's own FP64 arithmetic, generalised to 3-D grids (nz > 1);
 * with nz == 1 it is the reference's 2-D depth-averaged path. Parity is pinned
 * against the reference itself: tests/golden/ holds fixtures produced by the
 * reference's unmodified sources run on the CPU (oracle/build_ref.sh), and
 * tests/test_oracle_golden.py checks this restatement against them.
 *
 * The API mirrors include/agb.h so a test drives the oracle and the CUDA engine
 * with the same descriptor and the same host buffers.
 */
#ifndef ORC_ORACLE_H
#define ORC_ORACLE_H

#include <stdint.h>

#include "../include/agb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_world orc_world;

int orc_world_create(const agb_world_desc* d, orc_world** out);
void orc_world_destroy(orc_world* w);
void orc_set_threads(int n);

int orc_world_spawn(orc_world* w, const agb_spawn* p);
int orc_world_spawn_seeded(orc_world* w, const agb_spawn* p, uint64_t seed);
int orc_world_set_light(orc_world* w, const agb_light* light);
int orc_world_set_flash(orc_world* w, int32_t active, double power);
int orc_world_spawn_taumoeba(orc_world* w, int32_t count, uint64_t seed);
int orc_world_import_taumoeba(orc_world* w, const agb_taumoeba* src, int32_t count, uint64_t next_id);
int orc_world_export_taumoeba(orc_world* w, agb_taumoeba* dst, int32_t max_count, int32_t* count, uint64_t* next_id);
int orc_world_flash_audit(orc_world* w, double* impulse_ns, double* discharged_j);
int orc_world_import_cells(orc_world* w, const agb_cells* src, int32_t count, uint64_t next_id);
int orc_world_export_cells(orc_world* w, agb_cells* dst, int32_t max_count, int32_t* count,
                           uint64_t* next_id);
int orc_world_import_field(orc_world* w, int32_t field, const float* src);
int orc_world_export_field(orc_world* w, int32_t field, float* dst);
int orc_world_export_deposit(orc_world* w, int32_t field, uint64_t* dst);
int orc_world_apply_brush(orc_world* w, int32_t kind, double x, double y, double radius, double strength);

int orc_world_step(orc_world* w, int32_t ticks);
int orc_world_stage(orc_world* w, int32_t stage);
int orc_world_diffuse(orc_world* w, int32_t field, double dt);
int orc_world_stats(orc_world* w, agb_stats* out);
int orc_world_stats_accum(orc_world* w, uint64_t out[12]);
int orc_world_set_clock(orc_world* w, double physics_rate, double biology_rate);
int orc_world_export_hash(orc_world* w, int32_t dims[4], uint32_t* keys_sorted, uint32_t* vals_sorted,
                          int32_t* bucket_start, int32_t* bucket_end);
int orc_world_export_forces(orc_world* w, double* fx, double* fy, double* fz);
int orc_world_export_term_scales(orc_world* w, double* force, double* vel, double* disp);
int orc_world_counters(orc_world* w, int64_t out[4]);

/* Known-answer hooks for the RNG (src/core/rng.cuh). */
void orc_pcg32_seed_draws(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t* out);
uint64_t orc_cell_rng_init(uint64_t seed, uint64_t id);
uint64_t orc_pcg_split(uint64_t parent_state, uint64_t daughter_id);

/* Snapshot bytes (header + body) and the FNV-1a hash of contracts/snapshot_v1.h. */
uint64_t orc_fnv1a64(const void* data, uint64_t n, uint64_t h);
int64_t orc_world_snapshot(orc_world* w, const char* scenario_id, char* out, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
