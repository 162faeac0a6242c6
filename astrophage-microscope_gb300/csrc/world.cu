// world.cu -- the C ABI (include/agb.h): world lifetime, import/export in
// contract layout, the tick sequence of world_step (src/sim/step.cu:109-184)
// and its CUDA-graph replay.
//
// The tick never synchronises with the host: population counts, division and
// compaction decisions live in device memory (DevState), so a tick -- or many
// ticks -- can be captured once and replayed as a single graph launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "world_impl.cuh"

using namespace agb;

namespace {

agb_status fail(agb_world* w, agb_status s, const std::string& what) {
    if (w) w->err = what;
    return s;
}

agb_status cuda_fail(agb_world* w, cudaError_t e, const char* what) {
    return fail(w, AGB_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

#define AGB_CUDA(w, call)                                       \
    do {                                                        \
        const cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail((w), _e, #call); \
    } while (0)

template <typename T>
cudaError_t dalloc(agb_world* w, T** p, size_t bytes) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, bytes ? bytes : 1);
    if (e == cudaSuccess) { w->allocs.push_back(q); *p = static_cast<T*>(q); }
    return e;
}

unsigned long long dkey_host(double v) {
    unsigned long long b;
    std::memcpy(&b, &v, 8);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

// One blob per SoA, 256-byte aligned arrays in contract order
// (src/sim/cell_store.cu:139-193).
SoA carve(void* blob, int32_t cap) {
    char* p = static_cast<char*>(blob);
    auto take = [&](size_t elem) { char* q = p; p += align256(elem * (size_t)cap); return q; };
    SoA v{};
    v.id = (uint64_t*)take(8); v.flags = (uint32_t*)take(4); v.death_cause = (uint8_t*)take(1);
    v.x = (double*)take(8); v.y = (double*)take(8); v.z = (double*)take(8);
    v.vx = (double*)take(8); v.vy = (double*)take(8); v.vz = (double*)take(8);
    v.energy = (double*)take(8); v.temp_cell = (float*)take(4); v.emit_power = (float*)take(4);
    v.dir_x = (float*)take(4); v.dir_y = (float*)take(4); v.dir_z = (float*)take(4);
    v.biomass = (double*)take(8); v.co2_held = (double*)take(8); v.age_s = (float*)take(4);
    v.rng_state = (uint64_t*)take(8); v.taxis_memory = (float*)take(4); v.run_timer = (float*)take(4);
    v.t_local = (float*)take(4); v.irradiance = (float*)take(4); v.co2_local = (float*)take(4);
    v.n2_local = (float*)take(4);
    return v;
}
size_t soa_bytes(int32_t cap) {
    const size_t sizes[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};
    size_t t = 0;
    for (size_t s : sizes) t += align256(s * (size_t)cap);
    return t;
}
void soa_arrays(const SoA& v, void* p[25]) {
    void* q[25] = {v.id, v.flags, v.death_cause, v.x, v.y, v.z, v.vx, v.vy, v.vz, v.energy,
                   v.temp_cell, v.emit_power, v.dir_x, v.dir_y, v.dir_z, v.biomass, v.co2_held,
                   v.age_s, v.rng_state, v.taxis_memory, v.run_timer, v.t_local, v.irradiance,
                   v.co2_local, v.n2_local};
    std::memcpy(p, q, sizeof(q));
}
void host_arrays(const agb_cells* h, void* p[25]) {
    void* q[25] = {h->id, h->flags, h->death_cause, h->x, h->y, h->z, h->vx, h->vy, h->vz,
                   h->energy, h->temp_cell, h->emit_power, h->dir_x, h->dir_y, h->dir_z,
                   h->biomass, h->co2_held, h->age_s, h->rng_state, h->taxis_memory,
                   h->run_timer, h->t_local, h->irradiance, h->co2_local, h->n2_local};
    std::memcpy(p, q, sizeof(q));
}
const size_t kElem[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};

float float_at_or_above(double v) {
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, INFINITY);
    return f;
}
float float_at_or_below(double v) {
    float f = (float)v;
    if ((double)f > v) f = std::nextafter(f, -INFINITY);
    return f;
}

// Stable substep count (src/fields/grid.cuh:51-53; 1/6 bound for 3-D).
int32_t substeps_for(const GridDev& g, double D, double dt) {
    const double lim = g.nz > 1 ? 6.0 : 4.0;
    return (int32_t)(dt / (g.dx * g.dx / (lim * D))) + 1;
}
bool coeff_ok(const GridDev& g, float c) { return g.nz > 1 ? c <= (float)(1.0 / 6.0) : c <= 0.25f; }

// ou_position_shape (integrator.cuh:80-91) on the host.
double ou_shape_host(double x) {
    if (x < 1.0e-2) {
        const double x3 = x * x * x;
        return x3 * (2.0 / 3.0 + x * (-0.5 + x * (7.0 / 30.0 + x * (-1.0 / 12.0))));
    }
    const double e = std::exp(-x);
    return 2.0 * x - 3.0 + 4.0 * e - e * e;
}

// The predator's per-world constants (predation.cu:80-158): the memory weight
// of tau_should_tumble, tau_drag at the ambient temperature, ou_coefficients
// of TAU_MASS (integrator.cuh:103-121) and the noise factors of
// ou_advance_axis, all in the reference's FP64 expressions; the walls.
void compute_tau_params(agb_world* w) {
    TauParams& q = w->taup;
    const TickParams& p = w->tp;
    q.dt = p.dt;
    q.dt_bio = p.dt_bio;
    q.dt_f = (float)q.dt;
    q.dt_bio_f = (float)q.dt_bio;
    q.alpha = -std::expm1(-q.dt / AGB_TAXIS_MEMORY_TIME);
    const double T = w->d.ambient_temp;
    q.gamma = 6.0 * AGB_PI * (AGB_VF_A * std::exp(AGB_VF_B / (T - AGB_VF_C))) * AGB_TAU_RADIUS;
    const double beta = q.gamma / AGB_TAU_MASS;
    const double x = beta * q.dt;
    q.ome = -std::expm1(-x);
    q.inv_beta = 1.0 / beta;
    const double kTm = AGB_K_BOLTZ * T / AGB_TAU_MASS;
    const double var_vv = kTm * (-std::expm1(-2.0 * x));
    const double var_rr = kTm * q.inv_beta * q.inv_beta * ou_shape_host(x);
    q.s_vv = std::sqrt(var_vv > 0.0 ? var_vv : 0.0);
    q.s_rr = std::sqrt(var_rr > 0.0 ? var_rr : 0.0);
    const double s_rv = kTm * q.inv_beta * q.ome * q.ome;
    q.noise_a = q.s_rr > 0.0 ? s_rv / q.s_rr : 0.0;
    const double b2 = q.s_vv * q.s_vv - q.noise_a * q.noise_a;
    q.noise_b = std::sqrt(b2 > 0.0 ? b2 : 0.0);
    const double ext[3] = {w->d.chamber_w, w->d.chamber_h, w->d.chamber_d};
    for (int a = 0; a < 3; ++a) {
        q.half[a] = 0.5 * ext[a];
        q.lo[a] = -q.half[a] + AGB_TAU_RADIUS;
        q.hi[a] = q.half[a] - AGB_TAU_RADIUS;
        q.span[a] = 2.0 * q.half[a];
    }
    q.boundary_x = w->d.boundary_x;
    q.boundary_y = w->d.boundary_y;
    q.noise = w->d.thermal_noise ? 1 : 0;
    q.disposition = w->d.store_disposition;
    q.compaction = w->d.tau_compaction_enabled ? 1 : 0;
}

agb_status compute_tick_params(agb_world* w) {
    TickParams& p = w->tp;
    const Ctx& c = w->c;
    p.dt = AGB_DT_PHYSICS * w->physics_rate;
    p.dt_inv = 1.0 / p.dt;
    p.dtf = (float)p.dt;
    p.k_contact = (float)(AGB_CONTACT_STIFFNESS / w->physics_rate);
    p.k_contact64 = AGB_CONTACT_STIFFNESS / w->physics_rate;
    p.k_trap = (float)(w->d.trap_stiffness / w->physics_rate);
    p.dt_bio = p.dt * w->biology_rate;
    p.dt_bio_f = (float)p.dt_bio;
    p.taxis_alpha = 1.0 - std::exp(-p.dt / AGB_TAXIS_MEMORY_TIME);     // taxis.cuh:38-41
    p.max_emit_power = w->d.max_emit_power > 0.0 ? w->d.max_emit_power : AGB_PETROVA_MAX_POWER;
    const GridDev& T = c.g[AGB_FIELD_TEMPERATURE];
    if (T.enabled) {
        const double D = w->d.grid[AGB_FIELD_TEMPERATURE].diffusivity;
        p.t_substeps = substeps_for(T, D, p.dt);
        p.t_dt_sub = p.dt / p.t_substeps;
        p.t_coeff = (float)(D * p.t_dt_sub / (T.dx * T.dx));
        if (!coeff_ok(T, p.t_coeff)) return fail(w, AGB_INVALID_ARGUMENT, "diffusion coefficient unstable");
        // thermal_step (src/sim/thermal.cu:86-90): capacity of one voxel of water.
        p.t_cap = AGB_WATER_DENSITY * AGB_WATER_SPECIFIC_HEAT * T.dx * T.dx * T.dz_eff;
        const double relax = -std::expm1(-AGB_CONDUCTION_COEFF * p.t_dt_sub / p.t_cap);
        p.t_relax = (float)relax;
        p.t_cap_relax = (float)(p.t_cap * relax);
    }
    for (int f : {AGB_FIELD_CO2, AGB_FIELD_N2}) {
        const GridDev& g = c.g[f];
        int32_t steps = 0;
        float coeff = 0.0f;
        if (g.enabled) {
            const double D = w->d.grid[f].diffusivity;
            steps = substeps_for(g, D, p.dt);
            coeff = (float)(D * (p.dt / steps) / (g.dx * g.dx));
            if (!coeff_ok(g, coeff)) return fail(w, AGB_INVALID_ARGUMENT, "diffusion coefficient unstable");
        }
        if (f == AGB_FIELD_CO2) { p.c_substeps = steps; p.c_coeff = coeff; }
        else { p.n_substeps = steps; p.n_coeff = coeff; }
    }
    compute_tau_params(w);
    return AGB_OK;
}

void compute_light(agb_world* w) {
    Ctx& c = w->c;
    const agb_light& L = w->d.light;
    double dx = L.dir_x, dy = L.dir_y, dz = L.dir_z;
    const double l = std::sqrt(dx * dx + dy * dy + dz * dz);          // normalize, vec.cuh:34-37
    if (l > 0.0) { dx *= 1.0 / l; dy *= 1.0 / l; dz *= 1.0 / l; }
    else { dx = 0.0; dy = 0.0; dz = 1.0; }
    c.ldx = dx; c.ldy = dy; c.ldz = dz;
    c.lx = (float)dx; c.ly = (float)dy; c.lz = (float)dz;
    const double ax = std::fabs(dx), ay = std::fabs(dy), az = std::fabs(dz);
    int axis = ax >= ay ? 0 : 1;                                      // emission.cu:161-163
    if (az > ax && az > ay) axis = 2;
    const double comp = axis == 0 ? dx : (axis == 1 ? dy : dz);
    c.light_axis = axis;
    c.light_sign = comp >= 0.0 ? 1 : -1;
    const int zeros = (c.lx == 0.0f) + (c.ly == 0.0f) + (c.lz == 0.0f);
    c.light_axis_exact = zeros == 2 ? axis : -1;
    c.source = L.enabled ? L.irradiance : 0.0f;
    c.source_d = (double)c.source;
    c.ambient_irr = L.ambient;
    const GridDev& I = c.g[AGB_FIELD_IRRADIANCE];
    c.face_area = axis == 2 ? I.dx * I.dx : I.dx * I.dz_eff;          // emission.cu:164
    const long long deps[4] = {c.stamp_alive, 2 * c.stamp_alive, 3 * c.stamp_alive, c.stamp_dead};
    for (int k = 0; k < 4; ++k) {
        c.occl_dep[k] = (unsigned long long)deps[k];
        c.occl_fac[k] = occlusion_of(deps[k], I.scale, c.face_area);
    }
}

float* field_value(agb_world* w, int f) { return w->gbuf[f][w->gcur[f]]; }

// The irradiance field changed outside the sweep: the next sweep rewrites
// every line (enqueued on s).
void irr_all_lines(agb_world* w, cudaStream_t s) {
    if (w->c.irr_marks) cudaMemsetAsync(w->c.irr_marks, 2, (size_t)w->irr_mark_bytes, s);
}

void refresh_grid_ptrs(agb_world* w) {
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) {
        w->c.g[f].value = w->gbuf[f][w->gcur[f]];
        w->c.g[f].scratch = w->gbuf[f][1 - w->gcur[f]];
    }
}

void ftcs(agb_world* w, int f, float coeff, cudaStream_t s) {
    refresh_grid_ptrs(w);
    const CUtensorMap* map = (w->use_tma && w->tmap_ok[f]) ? &w->tmap[f][w->gcur[f]] : nullptr;
    launch_ftcs(w->c.g[f], field_value(w, f), w->gbuf[f][1 - w->gcur[f]], coeff, w->gbc[f], w->gface[f],
                w->grobin[f], map, &w->tplan[f], &w->S->error, s);
    w->gcur[f] = 1 - w->gcur[f];
    refresh_grid_ptrs(w);
}

// Stage bodies (src/sim/step.cu:109-184 and the functions it calls).
void stage_hash(agb_world* w, cudaStream_t s) {
    hash_build(w->S, w->c.h, w->c.capacity, w->kalt, w->valt, w->hist, w->blocks, s);
}

void stage_thermal(agb_world* w, cudaStream_t s) {   // thermal_step, src/sim/thermal.cu:75-103
    if (!w->c.g[AGB_FIELD_TEMPERATURE].enabled) return;
    for (int32_t k = 0; k < w->tp.t_substeps; ++k) {
        refresh_grid_ptrs(w);
        if (w->d.thermal_enabled) {
            launch_thermal(w->S, w->c, w->tp, w->blocks, k == 0, s);
            launch_flush_by_cells(w->S, w->c.g[AGB_FIELD_TEMPERATURE], nullptr, w->blocks, s, true, w->c.t_vox);
        }
        ftcs(w, AGB_FIELD_TEMPERATURE, w->tp.t_coeff, s);
    }
}

bool emission_active(const agb_world* w) {
    return w->d.emission_enabled && w->c.g[AGB_FIELD_IRRADIANCE].enabled &&
           (w->c.source > 0.0f || w->c.ambient_irr > 0.0f);
}

void stage_emission(agb_world* w, cudaStream_t s) {  // emission_step, src/sim/emission.cu:119-177
    if (!w->c.g[AGB_FIELD_IRRADIANCE].enabled) return;
    if (w->c.source <= 0.0f && w->c.ambient_irr <= 0.0f) return;
    refresh_grid_ptrs(w);
    launch_emission(w->S, w->c, w->tp, w->stamp_idx, w->occl_factor, w->c.source > 0.0f, w->blocks,
                    w->walk_lanes, s);
}

void stage_motion(agb_world* w, cudaStream_t s) {    // motion_step, src/sim/integrator.cu:154-177
    refresh_grid_ptrs(w);
    launch_motion(w->S, w->c, w->tp, w->fx, w->fy, w->fz, w->blocks, w->walk_lanes, s);
}

// src/sim/step.cu:168-171. The flushes there are no-ops here by construction:
// the only CO2 depositor (uptake) flushes its own deposits, and nothing
// deposits into N2 without predators.
void stage_slow_fields(agb_world* w, cudaStream_t s) {
    if (w->c.g[AGB_FIELD_CO2].enabled)
        for (int32_t k = 0; k < w->tp.c_substeps; ++k) ftcs(w, AGB_FIELD_CO2, w->tp.c_coeff, s);
    if (w->c.g[AGB_FIELD_N2].enabled)
        for (int32_t k = 0; k < w->tp.n_substeps; ++k) ftcs(w, AGB_FIELD_N2, w->tp.n_coeff, s);
}

// Stage 9b or 3: the flash when armed, else taxis when enabled (step.cu:158-162).
void stage_flash_or_taxis(agb_world* w, cudaStream_t s) {
    if (w->flash_active) launch_flash(w->S, w->tp.dt, w->flash_power, w->flash_accum, w->blocks, s);
    else if (w->d.taxis_enabled) launch_taxis(w->S, w->c, w->tp, w->blocks, s);
}

// predation_step (predation.cu:434-484) once predators have been placed: it
// senses this tick's cell hash and the N2 as diffused this tick.
void stage_predation(agb_world* w, cudaStream_t s) {
    if (!w->tau_active) return;
    refresh_grid_ptrs(w);
    launch_predation(w->tS, w->S, w->c.h, w->c.g[AGB_FIELD_N2], w->taup, w->claim, w->c.capacity, w->tau_cap, s);
}

bool compaction_allowed(const agb_world* w) {
    const int32_t P = w->d.compaction_period > 0 ? w->d.compaction_period : 1;
    return w->d.compaction_enabled && ((w->tick + 1) % (uint64_t)P) == 0;
}

void stage_lifecycle(agb_world* w, cudaStream_t s, bool demand_done = false) {  // src/sim/lifecycle.cu:208-294
    refresh_grid_ptrs(w);
    launch_lifecycle(w->S, w->c, w->tp, w->life, compaction_allowed(w), w->blocks, s, demand_done);
}

void stage_clock(agb_world* w) {
    ++w->tick;
    w->sim_time += w->tp.dt;
}

// One tick as a small DAG. The irradiance field (stamps, occlusion factors,
// sweep) reads the cells as thermal leaves them but not the hash; the last
// thermal substep's flush and FTCS pass touch only the temperature grid; the
// CO2/N2 diffusion touches only those grids. So three side streams -- branches
// of the captured graph -- run them beside the hash build, joined where the
// reference's order needs their results: the irradiance field and the
// diffused temperature before the per-cell pass (feeding walks the hash,
// forces sample T), the slow fields before integration, which also enters
// the lifecycle's CO2 demand from the diffused CO2 (uptake reads it too).
// Motion samples CO2 and N2 from the buffers as they were before this tick's
// diffusion, exactly as in src/sim/step.cu:164-171, while the diffusion
// writes the other ping-pong buffer.
void tick_surrogate(agb_world* w, cudaStream_t s);

// A section timer mark (start = 0, end = 1) on stream s when timing is on;
// an external event record, so that stream capture keeps it as a graph node.
static void mark(agb_world* w, int section, int end, cudaStream_t s) {
    if (w->timing) cudaEventRecordWithFlags(w->tev[2 * section + end], s, cudaEventRecordExternal);
}

void tick_once(agb_world* w, cudaStream_t s) {
    if (w->sg) { tick_surrogate(w, s); return; }
    cudaStream_t s1 = w->side[0], s2 = w->side[1], s3 = w->side[2];
    mark(w, AGB_SECTION_TICK, 0, s);
    cudaEventRecord(w->ev[0], s);
    cudaStreamWaitEvent(s1, w->ev[0], 0);
    cudaStreamWaitEvent(s2, w->ev[0], 0);
    // thermal_step (thermal.cu:75-103): all substeps on s1 except the last
    // one's flush and FTCS pass, which fork onto s3 once its thermal kernel
    // has run.
    const bool thermal = w->d.thermal_enabled && w->c.g[AGB_FIELD_TEMPERATURE].enabled;
    const int32_t nsub = thermal ? w->tp.t_substeps : 0;
    if (nsub > 0) mark(w, AGB_SECTION_THERMAL, 0, s1);
    for (int32_t k = 0; k < nsub; ++k) {
        refresh_grid_ptrs(w);
        launch_thermal(w->S, w->c, w->tp, w->blocks, k == 0, s1);
        if (k + 1 == nsub) break;
        launch_flush_by_cells(w->S, w->c.g[AGB_FIELD_TEMPERATURE], nullptr, w->blocks, s1, true, w->c.t_vox);
        ftcs(w, AGB_FIELD_TEMPERATURE, w->tp.t_coeff, s1);
    }
    if (nsub > 0) mark(w, AGB_SECTION_THERMAL, 1, s1);
    cudaEventRecord(w->ev[3], s1);
    cudaStreamWaitEvent(s3, w->ev[3], 0);
    if (nsub > 0) {
        mark(w, AGB_SECTION_T_DIFFUSE, 0, s3);
        launch_flush_by_cells(w->S, w->c.g[AGB_FIELD_TEMPERATURE], nullptr, w->blocks, s3, true, w->c.t_vox);
        ftcs(w, AGB_FIELD_TEMPERATURE, w->tp.t_coeff, s3);
        mark(w, AGB_SECTION_T_DIFFUSE, 1, s3);
    }
    cudaEventRecord(w->ev[4], s3);
    const bool emit = emission_active(w);
    if (emit) {
        refresh_grid_ptrs(w);
        mark(w, AGB_SECTION_IRRADIANCE, 0, s1);
        launch_emission_prep(w->S, w->c, w->tp, w->stamp_idx, w->occl_factor, w->c.source > 0.0f, w->blocks, s1);
        mark(w, AGB_SECTION_IRRADIANCE, 1, s1);
    }
    cudaEventRecord(w->ev[1], s1);
    refresh_grid_ptrs(w);
    const Ctx pre = w->c;                       // CO2/N2 as motion must see them
    mark(w, AGB_SECTION_SLOW_FIELDS, 0, s2);
    stage_slow_fields(w, s2);
    mark(w, AGB_SECTION_SLOW_FIELDS, 1, s2);
    cudaEventRecord(w->ev[2], s2);
    mark(w, AGB_SECTION_HASH, 0, s);
    stage_hash(w, s);
    mark(w, AGB_SECTION_HASH, 1, s);
    cudaStreamWaitEvent(s, w->ev[1], 0);
    cudaStreamWaitEvent(s, w->ev[4], 0);
    mark(w, AGB_SECTION_CELL_PASS, 0, s);
    // Feeding, taxis (step.cu:161-162) and forces: one kernel per cell pass,
    // or the three passes in turn. Feeding reads only the irradiance grid.
    Ctx c = w->c;
    for (int f : {AGB_FIELD_CO2, AGB_FIELD_N2}) c.g[f] = pre.g[f];
    // While the spin-drive flash is armed it replaces taxis (step.cu:158-162);
    // those ticks take the three passes in turn.
    if (w->fuse_cells && !w->flash_active) {
        launch_cell_step(w->S, c, w->tp, w->fx, w->fy, w->fz, w->blocks, w->walk_lanes, emit,
                         w->d.taxis_enabled != 0, s);
    } else {
        if (emit) launch_feed(w->S, w->c, w->tp, w->blocks, w->walk_lanes, s);
        stage_flash_or_taxis(w, s);
        launch_forces(w->S, c, w->tp, w->fx, w->fy, w->fz, w->blocks, w->walk_lanes, s);
    }
    mark(w, AGB_SECTION_CELL_PASS, 1, s);
    cudaStreamWaitEvent(s, w->ev[2], 0);
    mark(w, AGB_SECTION_INTEGRATE, 0, s);
    const GridDev& co2 = w->c.g[AGB_FIELD_CO2];
    const double gv = co2.enabled ? co2.dx * co2.dx * co2.dz_eff : 0.0;
    // With predators the CO2 demand waits for predation (it kills prey before
    // the lifecycle books demand, step.cu:173-180); otherwise integration
    // books it.
    const bool fuse_demand = co2.enabled && !w->tau_active;
    launch_integrate(w->S, c, w->tp, w->fx, w->fy, w->fz, w->blocks, co2,
                     fuse_demand ? w->life.co2_demand : nullptr, gv, w->life.co2_want, w->life.co2_vox, s);
    mark(w, AGB_SECTION_INTEGRATE, 1, s);
    mark(w, AGB_SECTION_LIFECYCLE, 0, s);
    stage_predation(w, s);
    stage_lifecycle(w, s, fuse_demand);
    mark(w, AGB_SECTION_LIFECYCLE, 1, s);
    mark(w, AGB_SECTION_TICK, 1, s);
    stage_clock(w);
}

// A tick while the learned surrogate drives the temperature and CO2 grids:
// the stages run as in tick_once, except that the cells' heat exchange
// accumulates in the temperature deposit grid instead of being flushed, and
// neither grid is diffused. Every sg_steps ticks the accumulated heat becomes
// a constant per-step source and the surrogate advances both grids by the
// whole window (its judge runs the plain FTCS window every judge_every-th
// call and takes over when the network is off by more than its tolerance).
// CO2 uptake is still folded into the grid every tick, so the window has no
// CO2 source. Cells see the grids as they stood at the start of the window.
void tick_surrogate(agb_world* w, cudaStream_t s) {
    refresh_grid_ptrs(w);
    stage_hash(w, s);
    if (w->d.thermal_enabled && w->c.g[AGB_FIELD_TEMPERATURE].enabled)
        for (int32_t k = 0; k < w->tp.t_substeps; ++k) launch_thermal(w->S, w->c, w->tp, w->blocks, k == 0, s);
    if (w->d.emission_enabled) stage_emission(w, s);
    stage_flash_or_taxis(w, s);
    launch_motion(w->S, w->c, w->tp, w->fx, w->fy, w->fz, w->blocks, w->walk_lanes, s);
    stage_predation(w, s);
    stage_lifecycle(w, s);
    stage_clock(w);
    if (w->tick % (uint64_t)w->sg_steps == 0) {
        const GridDev& T = w->c.g[AGB_FIELD_TEMPERATURE];
        surrogate_source_from_deposit(w->gdep[AGB_FIELD_TEMPERATURE], w->sg_q, T.count, 1.0 / T.scale, w->sg_steps, s);
        agb_surrogate_advance(w->sg, field_value(w, AGB_FIELD_TEMPERATURE), field_value(w, AGB_FIELD_CO2), w->sg_q,
                              nullptr, 0, nullptr, s);
    }
}

uint32_t parity_bits(const agb_world* w) {
    uint32_t p = 0;
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) p |= (uint32_t)w->gcur[f] << f;
    return p;
}

void invalidate_graphs(agb_world* w) {
    for (auto& g : w->graphs) cudaGraphExecDestroy(g.exec);
    w->graphs.clear();
    ++w->version;
}

// Host <-> device cell transfer through device-accessible host memory
// (pinned, or any memory on a system where the GPU reads host page tables,
// e.g. Grace over NVLink-C2C): one kernel gathers or scatters all 25 arrays
// in contract layout, instead of 25 copies and a state round trip.
struct HostCells { void* p[25]; };

__device__ __forceinline__ void soa_ptrs_dev(const SoA& v, void* p[25]) {
    p[0] = v.id; p[1] = v.flags; p[2] = v.death_cause; p[3] = v.x; p[4] = v.y; p[5] = v.z; p[6] = v.vx;
    p[7] = v.vy; p[8] = v.vz; p[9] = v.energy; p[10] = v.temp_cell; p[11] = v.emit_power; p[12] = v.dir_x;
    p[13] = v.dir_y; p[14] = v.dir_z; p[15] = v.biomass; p[16] = v.co2_held; p[17] = v.age_s;
    p[18] = v.rng_state; p[19] = v.taxis_memory; p[20] = v.run_timer; p[21] = v.t_local;
    p[22] = v.irradiance; p[23] = v.co2_local; p[24] = v.n2_local;
}

// One thread per cell: every load of the cell's 25 elements is issued before
// the first store, so each thread keeps up to 25 requests in flight over the
// host link instead of one round trip per array. Null `pres` entries (arrays
// the caller left out) are skipped.
__device__ __forceinline__ void move_cell(void* const* dst, const void* const* src, const void* const* pres,
                                          int64_t i) {
    constexpr uint8_t E[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};
    uint64_t v[25];
#pragma unroll
    for (int k = 0; k < 25; ++k) {
        v[k] = 0;
        if (pres[k]) {
            if (E[k] == 8) v[k] = static_cast<const uint64_t*>(src[k])[i];
            else if (E[k] == 4) v[k] = static_cast<const uint32_t*>(src[k])[i];
            else v[k] = static_cast<const uint8_t*>(src[k])[i];
        }
    }
#pragma unroll
    for (int k = 0; k < 25; ++k) {
        if (pres[k]) {
            if (E[k] == 8) static_cast<uint64_t*>(dst[k])[i] = v[k];
            else if (E[k] == 4) static_cast<uint32_t*>(dst[k])[i] = (uint32_t)v[k];
            else static_cast<uint8_t*>(dst[k])[i] = (uint8_t)v[k];
        }
    }
}

constexpr int kXferThreads = 128;

__global__ void __launch_bounds__(kXferThreads) cells_import_kernel(DevState* S, HostCells h, int32_t count,
                                                                    uint64_t next_id) {
    void* d[25];
    soa_ptrs_dev(S->cur, d);
    const int64_t st = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += st)
        move_cell(d, h.p, h.p, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) { S->count = count; S->next_id = next_id; }
}

__global__ void __launch_bounds__(kXferThreads) cells_export_kernel(DevState* S, HostCells h, int32_t max_count,
                                                                    int64_t* out) {
    void* d[25];
    soa_ptrs_dev(S->cur, d);
    const int32_t n = S->count < max_count ? S->count : max_count;
    const int64_t st = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += st)
        move_cell(h.p, d, h.p, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) { out[0] = S->count; out[1] = (int64_t)S->next_id; }
}

static unsigned xfer_blocks(int64_t n) {
    const int64_t b = (n + kXferThreads - 1) / kXferThreads;
    return (unsigned)(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

// True when the GPU can address every non-null host array directly and each
// is aligned to its element size (the kernels move whole elements; arrays
// packed end to end, as in a snapshot body, can start mid-element and take
// the copy path). The answer for the last pointer set is cached (a loop
// passes the same buffers).
bool host_cells_direct(agb_world* w, void* const hst[25]) {
    for (int k = 0; k < 25; ++k)
        if (hst[k] && (reinterpret_cast<uintptr_t>(hst[k]) % kElem[k]) != 0) return false;
    bool same = true;
    for (int k = 0; k < 25; ++k) same = same && w->direct_ptrs[k] == hst[k];
    if (same) return w->direct_ok;
    static int pageable = -1;
    if (pageable < 0) {
        int a = 0, b = 0;
        cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, w->dev);
        cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, w->dev);
        pageable = (a && b) ? 1 : 0;
    }
    bool ok = true;
    for (int k = 0; k < 25 && ok; ++k) {
        if (!hst[k]) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, hst[k]) != cudaSuccess) { cudaGetLastError(); ok = false; break; }
        ok = at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged ||
             (at.type == cudaMemoryTypeUnregistered && pageable == 1);
    }
    for (int k = 0; k < 25; ++k) w->direct_ptrs[k] = hst[k];
    w->direct_ok = ok;
    return ok;
}

agb_status read_state(agb_world* w, DevState& out, cudaStream_t s) {
    AGB_CUDA(w, cudaMemcpyAsync(&out, w->S, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

}  // namespace

// Entry points for the batch (batch.cu); see world_impl.cuh.
namespace agb {

void world_tick(agb_world* w, cudaStream_t s) { tick_once(w, s); }
void world_refresh(agb_world* w) { refresh_grid_ptrs(w); }
bool world_emission_active(const agb_world* w) { return emission_active(w); }
bool world_compaction_allowed(const agb_world* w) { return compaction_allowed(w); }
uint32_t world_parity(const agb_world* w) { return parity_bits(w); }
void world_set_parity(agb_world* w, uint32_t bits) {
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) w->gcur[f] = (bits >> f) & 1;
    refresh_grid_ptrs(w);
}
uint64_t world_phase(const agb_world* w) {
    const uint64_t P = w->d.compaction_period > 0 ? (uint64_t)w->d.compaction_period : 1;
    return w->tick % P;
}
void world_advance_clock(agb_world* w, int32_t ticks) {
    w->tick += (uint64_t)ticks;
    w->sim_time += w->tp.dt * ticks;
}
void world_set_clock_state(agb_world* w, uint64_t tick, double sim_time) {
    invalidate_graphs(w);
    w->tick = tick;
    w->sim_time = sim_time;
}

bool world_set_tiling(agb_world* w, int f, const FtcsPlan& p) {
    const GridDev& g = w->c.g[f];
    if (!g.enabled || g.nz <= 1 || !w->tmap_ok[f]) return false;
    CUtensorMap m[2];
    if (!make_plane_map(&m[0], w->gbuf[f][0], g.nx, g.ny, g.nz, p) ||
        !make_plane_map(&m[1], w->gbuf[f][1], g.nx, g.ny, g.nz, p))
        return false;
    w->tmap[f][0] = m[0];
    w->tmap[f][1] = m[1];
    w->tplan[f] = p;
    invalidate_graphs(w);
    return true;
}

float world_time_passes(agb_world* w, int f, int passes, cudaStream_t s) {
    const GridDev& g = w->c.g[f];
    if (!g.enabled || passes <= 0) return -1.0f;
    const float coeff = (float)(1.0 / 8.0);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1.0f;
    for (int k = 0; k < 2 * passes; ++k) ftcs(w, f, coeff, s);      // even: buffers end where they began
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess) return -1.0f;
    const bool ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    cudaGraphDestroy(graph);
    if (!ok) return -1.0f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = -1.0f;
    for (int r = 0; r < 4; ++r) {
        cudaEventRecord(e0, s);
        cudaGraphLaunch(exec, s);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) { best = -1.0f; break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && (best < 0.0f || ms < best)) best = ms;       // first replay warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(exec);
    return best < 0.0f ? best : best / (2.0f * passes);
}

}  // namespace agb

extern "C" {

void agb_world_desc_default(agb_world_desc* d) {
    std::memset(d, 0, sizeof(*d));
    d->abi_version = AGB_ABI_VERSION;
    d->chamber_w = AGB_CHAMBER_W;
    d->chamber_h = AGB_CHAMBER_H;
    d->chamber_d = AGB_CHAMBER_D;
    d->capacity = AGB_DEFAULT_CELLS;
    d->seed = 20260802ull;
    d->boundary_x = d->boundary_y = AGB_WALL_REFLECTING;
    d->gravity_axis = AGB_GRAVITY_Y;
    d->thermal_noise = d->contact_enabled = d->adhesion_enabled = d->thermal_enabled = 1;
    d->emission_enabled = d->taxis_enabled = d->occlusion_exact = 1;
    d->compaction_enabled = 0;
    d->store_disposition = AGB_STORE_VOID;
    d->ambient_temp = AGB_AMBIENT_TEMP_DEFAULT;
    const struct { int n; double D, init, scale; int bc; } g[4] = {
        {AGB_FIELD_N_TEMP, AGB_WATER_THERMAL_DIFFUSIVITY, AGB_AMBIENT_TEMP_DEFAULT, AGB_DEPOSIT_SCALE_TEMPERATURE, AGB_BC_ROBIN},
        {AGB_FIELD_N_CO2, AGB_CO2_DIFFUSIVITY_WATER, 0.0, AGB_DEPOSIT_SCALE_CO2, AGB_BC_NEUMANN},
        {AGB_FIELD_N_N2, AGB_N2_DIFFUSIVITY, 0.0, AGB_DEPOSIT_SCALE_N2, AGB_BC_NEUMANN},
        {AGB_FIELD_N_IRRAD, AGB_IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, AGB_DEPOSIT_SCALE_IRRADIANCE, AGB_BC_NEUMANN}};
    for (int f = 0; f < 4; ++f) {
        d->grid[f].nx = d->grid[f].ny = g[f].n;
        d->grid[f].nz = 1;
        for (int k = 0; k < 6; ++k) { d->grid[f].bc[k] = g[f].bc; d->grid[f].face_value[k] = g[f].init; }
        d->grid[f].diffusivity = g[f].D;
        d->grid[f].init = g[f].init;
        d->grid[f].deposit_scale = g[f].scale;
    }
    d->hash_cell_size = AGB_HASH_CELL_FACTOR * AGB_CELL_DIAMETER;
    d->light.dir_x = 1.0f;
    d->physics_rate = 1.0;
    d->biology_rate = 1.0;
    d->co2_mass_per_division = AGB_CO2_MASS_PER_DIVISION;
    d->max_emit_power = AGB_PETROVA_MAX_POWER;
    d->division_predicate = AGB_DIVIDE_CO2_QUOTA;
    d->compaction_period = 1;
    d->trap_slot = -1;
    d->tau_capacity = 0;
    d->tau_compaction_enabled = 0;
}

const char* agb_status_str(agb_status s) {
    static const char* names[] = {"Ok", "OutOfMemory", "CudaError", "InvalidArgument", "NotFound",
                                  "ParseError", "ContractVersionMismatch", "CapacityExceeded",
                                  "FileIoError", "Unsupported", "DeviceTimeout"};
    return (s >= 0 && s <= 10) ? names[s] : "Unknown";
}

const char* agb_last_error(const agb_world* w) { return w ? w->err.c_str() : ""; }

agb_status agb_device_info(int32_t* device, int32_t* sm_version, int32_t* sm_count) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AGB_CUDA_ERROR;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return AGB_CUDA_ERROR;
    if (device) *device = dev;
    if (sm_version) *sm_version = p.major * 10 + p.minor;
    if (sm_count) *sm_count = p.multiProcessorCount;
    return AGB_OK;
}

void agb_world_destroy(agb_world* w) {
    if (!w) return;
    invalidate_graphs(w);
    if (w->own_stream) cudaStreamDestroy(w->own_stream);
    for (cudaStream_t& st : w->side) if (st) cudaStreamDestroy(st);
    for (cudaEvent_t& e : w->ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t& e : w->tev) if (e) cudaEventDestroy(e);
    for (void* p : w->allocs) cudaFree(p);
    if (w->xfer_host) cudaFreeHost(w->xfer_host);
    delete w;
}

agb_status agb_world_create(const agb_world_desc* d, agb_world** out) {
    if (!out) return AGB_INVALID_ARGUMENT;
    *out = nullptr;
    if (!d || d->abi_version != AGB_ABI_VERSION) return AGB_CONTRACT_VERSION_MISMATCH;
    if (d->capacity <= 0 || d->capacity > AGB_MAX_CELLS) return AGB_INVALID_ARGUMENT;
    if (!(d->chamber_w > 0 && d->chamber_h > 0 && d->chamber_d > 0) || d->chamber_w > 0.4 ||
        d->chamber_h > 0.4 || d->chamber_d > 0.4)
        return AGB_INVALID_ARGUMENT;
    agb_world* w = new (std::nothrow) agb_world();
    if (!w) return AGB_OUT_OF_MEMORY;
    // AGB_PLAIN_STENCIL=1 selects the plain 3-D stencil (for A/B checks of the TMA one).
    if (const char* e = std::getenv("AGB_PLAIN_STENCIL")) w->use_tma = (e[0] != '1');
    w->d = *d;
    w->physics_rate = d->physics_rate;
    w->biology_rate = d->biology_rate;
    if (cudaGetDevice(&w->dev) != cudaSuccess) { delete w; return AGB_CUDA_ERROR; }
    cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, w->dev);
    const int32_t cap = d->capacity;
    {
        const int64_t b = (cap + 255) / 256;
        const int64_t lim = (int64_t)(w->sm_count > 0 ? w->sm_count : 1) * 8;
        w->blocks = (int32_t)(b < lim ? b : lim);
        // Neighbour walks. Populations of up to about 512 cells per SM run
        // feeding, taxis and forces as one kernel with one walk per cell (a
        // shorter dependent chain per tick), two lanes per cell; larger ones
        // keep separate kernels (lower register pressure, and feeding's walk
        // can skip the downstream layer), one thread per cell. Measured on
        // GB300 per tick: 25k cells 88.6 us (fused, 2 lanes) vs 98.8
        // (separate, 1 lane); 1M cells 1.47 ms (separate, 1 lane) vs 1.53
        // (fused, 1 lane) and 1.74 (fused, 2 lanes).
        const bool small = (int64_t)cap <= (int64_t)(w->sm_count > 0 ? w->sm_count : 1) * 512;
        w->walk_lanes = small ? 2 : 1;
        w->fuse_cells = small;
    }
    Ctx& c = w->c;
    c.chamber_w = d->chamber_w; c.chamber_h = d->chamber_h; c.chamber_d = d->chamber_d;
    c.capacity = cap;
    c.seed = d->seed;
    c.boundary_x = d->boundary_x; c.boundary_y = d->boundary_y; c.gravity_axis = d->gravity_axis;
    c.thermal_noise = d->thermal_noise; c.contact_enabled = d->contact_enabled;
    c.adhesion_enabled = d->adhesion_enabled; c.occlusion_exact = d->occlusion_exact;
    c.store_disposition = d->store_disposition; c.division_predicate = d->division_predicate;
    c.division_energy = d->division_energy;
    c.co2_quota = d->co2_mass_per_division;
    c.trap_slot = d->trap_slot; c.trap_x = d->trap_x; c.trap_y = d->trap_y;
    const double halves[3] = {0.5 * d->chamber_w, 0.5 * d->chamber_h, 0.5 * d->chamber_d};
    for (int a = 0; a < 3; ++a) {
        c.half[a] = halves[a];
        c.lo[a] = -halves[a] + AGB_CELL_RADIUS;
        c.hi[a] = halves[a] - AGB_CELL_RADIUS;
        c.lo_key[a] = dkey_host(c.lo[a]);
        c.hi_key[a] = dkey_host(c.hi[a]);
    }
    c.stamp_alive = std::llround(AGB_CELL_CROSS_SECTION * AGB_DEPOSIT_SCALE_IRRADIANCE);
    c.stamp_dead = std::llround(AGB_CELL_CROSS_SECTION * (1.0 - AGB_CELL_ALBEDO_DEAD) * AGB_DEPOSIT_SCALE_IRRADIANCE);
    c.setpoint_up = float_at_or_above(AGB_CELL_TEMP_SETPOINT);
    c.setpoint_hi = (float)AGB_CELL_TEMP_SETPOINT;
    c.setpoint_lo = (float)(AGB_CELL_TEMP_SETPOINT - (double)c.setpoint_hi);
    c.lethal_f = float_at_or_below(AGB_CELL_LETHAL_TEMP);
    c.stick_bits = (uint64_t)std::ceil(AGB_WALL_STICKINESS * 9007199254740992.0);

    // Fields (grid_create, src/fields/diffuse.cu:91-119).
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) {
        const agb_grid_desc& gd = d->grid[f];
        GridDev& g = c.g[f];
        std::memset(&g, 0, sizeof(g));
        if (gd.nx <= 0) continue;
        if (gd.nx <= 1 || gd.ny <= 1 || gd.nz < 1) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
        g.enabled = 1;
        g.nx = gd.nx; g.ny = gd.ny; g.nz = gd.nz;
        g.count = (int64_t)gd.nx * gd.ny * gd.nz;
        g.dx = d->chamber_w / (double)gd.nx;
        g.dz_eff = d->chamber_d / (double)gd.nz;
        if (gd.nz > 1 && std::fabs(g.dz_eff / g.dx - 1.0) > 1e-9) { agb_world_destroy(w); return AGB_UNSUPPORTED; }
        g.dxf = (float)g.dx;
        g.dzf = gd.nz > 1 ? (float)g.dz_eff : 0.0f;
        g.hx = 0.5f * gd.nx * g.dxf;
        g.hy = 0.5f * gd.ny * g.dxf;
        g.hz = 0.5f * gd.nz * g.dzf;
        g.scale = gd.deposit_scale;
        g.inv_scale_f = (float)(1.0 / gd.deposit_scale);
        g.inv_scale_lo = (float)(1.0 / gd.deposit_scale - (double)g.inv_scale_f);
        g.scale_f = (float)g.scale;
        g.vol_inv = 1.0 / (g.dx * g.dx * g.dz_eff);
        g.scale_inv = 1.0 / g.scale;
        for (int k = 0; k < 6; ++k) { w->gbc[f][k] = gd.bc[k]; w->gface[f][k] = (float)gd.face_value[k]; }
        w->grobin[f] = (float)(g.dx * AGB_AIR_CONVECTION_H / AGB_WATER_CONDUCTIVITY);
        for (int b = 0; b < 2; ++b)
            if (dalloc(w, &w->gbuf[f][b], sizeof(float) * g.count) != cudaSuccess) {
                agb_world_destroy(w); return AGB_OUT_OF_MEMORY;
            }
        if (dalloc(w, &w->gdep[f], sizeof(unsigned long long) * g.count) != cudaSuccess ||
            cudaMemset(w->gdep[f], 0, sizeof(unsigned long long) * g.count) != cudaSuccess) {
            agb_world_destroy(w); return AGB_OUT_OF_MEMORY;
        }
        g.deposit = w->gdep[f];
        if (g.nz > 1) w->tplan[f] = ftcs_plan(g.nx, g.ny, g.nz);
        w->tmap_ok[f] = g.nz > 1 && make_plane_map(&w->tmap[f][0], w->gbuf[f][0], g.nx, g.ny, g.nz, w->tplan[f]) &&
                        make_plane_map(&w->tmap[f][1], w->gbuf[f][1], g.nx, g.ny, g.nz, w->tplan[f]);
        launch_fill(w->gbuf[f][0], g.count, (float)gd.init, nullptr);
        launch_fill(w->gbuf[f][1], g.count, (float)gd.init, nullptr);
    }
    refresh_grid_ptrs(w);
    compute_light(w);

    // Hash (hash_create, src/sim/hash.cu:46-80).
    HashDev& h = c.h;
    const double cell = d->hash_cell_size > 0.0 ? d->hash_cell_size : AGB_HASH_CELL_FACTOR * AGB_CELL_DIAMETER;
    h.nx = std::max(1, (int32_t)std::ceil(d->chamber_w / cell));
    h.ny = std::max(1, (int32_t)std::ceil(d->chamber_h / cell));
    h.nz = std::max(1, (int32_t)std::ceil(d->chamber_d / cell));
    if ((double)h.nx * h.ny * h.nz >= 2147483647.0) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
    h.buckets = h.nx * h.ny * h.nz;
    h.cellf = (float)cell;
    h.inv = (float)(1.0 / cell);
    h.ox = (float)(-0.5 * h.nx * cell);
    h.oy = (float)(-0.5 * h.ny * cell);
    h.oz = (float)(-0.5 * h.nz * cell);
    // |FP32 bucket coordinate - FP64 one| <= ~3 * 2^-24 * n; twice that margin.
    h.margin = (float)(4.0e-7 * std::max(h.nx, std::max(h.ny, h.nz)) + 1.0e-6);
    // Fixed-point exponent: the largest K with |x| * 2^K < 2^62 over the chamber.
    {
        const double half = 0.5 * std::max(d->chamber_w, std::max(d->chamber_h, d->chamber_d));
        h.fix_k = 62 - (int32_t)std::ceil(std::log2(half));
        h.fix_inv = std::ldexp(1.0, -h.fix_k);
        h.fix_inv_f = (float)h.fix_inv;
        const float org[3] = {h.ox, h.oy, h.oz};
        for (int a = 0; a < 3; ++a) h.org_fix[a] = std::llround(std::ldexp((double)org[a], h.fix_k));
        h.cell_fix = std::llround(std::ldexp(cell, h.fix_k));
        h.cell_f = (float)std::ldexp((double)h.cell_fix, -h.fix_k);
    }
    if (h.nx > 2047 || h.ny > 2047 || h.nz > 1023) { agb_world_destroy(w); return AGB_UNSUPPORTED; }
    const size_t n = (size_t)cap;
    bool ok = dalloc(w, &h.keys, 4 * n) == cudaSuccess && dalloc(w, &h.vals, 4 * n) == cudaSuccess &&
              dalloc(w, &h.keys_sorted, 4 * n) == cudaSuccess && dalloc(w, &h.vals_sorted, 4 * n) == cudaSuccess &&
              dalloc(w, &w->kalt, 4 * n) == cudaSuccess && dalloc(w, &w->valt, 4 * n) == cudaSuccess &&
              dalloc(w, &w->hist, 4 * hash_sort_scratch_words(cap)) == cudaSuccess &&
              dalloc(w, &h.ranges, 8 * (size_t)h.buckets) == cudaSuccess &&
              dalloc(w, &h.occ, 4 * (((size_t)h.buckets + 31) / 32 + 1)) == cudaSuccess &&
              dalloc(w, &h.rec, 16 * n) == cudaSuccess;
    h.keys_prev = nullptr;
    // Cells: two SoA blobs (live + compaction target).
    w->blob_bytes = soa_bytes(cap);
    ok = ok && dalloc(w, &w->blob[0], w->blob_bytes) == cudaSuccess &&
         dalloc(w, &w->blob[1], w->blob_bytes) == cudaSuccess;
    const int32_t stiles = (cap + 1023) / 1024;
    ok = ok && dalloc(w, &w->life.flags, 4 * n) == cudaSuccess && dalloc(w, &w->life.prefix, 4 * n) == cudaSuccess &&
         dalloc(w, &w->life.tile_sums, 4 * (size_t)stiles) == cudaSuccess &&
         dalloc(w, &w->life.src, 4 * n) == cudaSuccess && dalloc(w, &w->life.co2_want, 8 * n) == cudaSuccess &&
         dalloc(w, &w->stamp_idx, 4 * n) == cudaSuccess && dalloc(w, &w->fx, 4 * n) == cudaSuccess &&
         dalloc(w, &w->fy, 4 * n) == cudaSuccess && dalloc(w, &w->fz, 4 * n) == cudaSuccess &&
         dalloc(w, &w->acc, 8 * 12) == cudaSuccess && dalloc(w, &w->S, sizeof(DevState)) == cudaSuccess;
    const int64_t irrn = c.g[AGB_FIELD_IRRADIANCE].enabled ? c.g[AGB_FIELD_IRRADIANCE].count : 1;
    ok = ok && dalloc(w, &w->occl_factor, 8 * (size_t)irrn) == cudaSuccess;
    if (c.g[AGB_FIELD_IRRADIANCE].enabled) {
        const GridDev& I = c.g[AGB_FIELD_IRRADIANCE];
        const int64_t yz = (int64_t)I.ny * I.nz, xz = (int64_t)I.nx * I.nz, xy = (int64_t)I.nx * I.ny;
        w->irr_mark_bytes = std::max(yz, std::max(xz, xy));
        ok = ok && dalloc(w, &c.irr_marks, (size_t)w->irr_mark_bytes) == cudaSuccess;
        w->irr_bit_words = (I.count + 31) / 32;
        ok = ok && dalloc(w, &c.irr_stamp_bits, 4 * (size_t)w->irr_bit_words) == cudaSuccess;
    }
    c.t_vox = nullptr;
    if (c.g[AGB_FIELD_TEMPERATURE].enabled && c.g[AGB_FIELD_TEMPERATURE].count <= INT32_MAX)
        ok = ok && dalloc(w, &c.t_vox, 4 * n) == cudaSuccess;
    w->life.co2_vox = nullptr;
    if (c.g[AGB_FIELD_CO2].enabled && c.g[AGB_FIELD_CO2].count <= INT32_MAX)
        ok = ok && dalloc(w, &w->life.co2_vox, 4 * n) == cudaSuccess;
    for (cudaStream_t& st : w->side) ok = ok && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t& e : w->ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    const int64_t co2n = c.g[AGB_FIELD_CO2].enabled ? c.g[AGB_FIELD_CO2].count : 1;
    ok = ok && dalloc(w, &w->life.co2_demand, 8 * (size_t)co2n) == cudaSuccess;
    ok = ok && dalloc(w, &w->flash_accum, 8 * 4) == cudaSuccess;
    // The predator store (taumoeba_create, predation.cu:306-418) and the per-cell claim words.
    w->tau_cap = d->tau_capacity > 0 ? d->tau_capacity : AGB_DEFAULT_TAUMOEBA;
    if (w->tau_cap > AGB_MAX_TAUMOEBA) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
    for (void*& b : w->tau_blob) ok = ok && dalloc(w, &b, tau_blob_bytes(w->tau_cap)) == cudaSuccess;
    ok = ok && dalloc(w, &w->tS, sizeof(TauState)) == cudaSuccess;
    ok = ok && dalloc(w, &w->claim, 8 * (size_t)cap) == cudaSuccess;
    if (!ok) { agb_world_destroy(w); return AGB_OUT_OF_MEMORY; }
    {
        TauState ts{};
        ts.cur = tau_carve(w->tau_blob[0], w->tau_cap);
        ts.spare = tau_carve(w->tau_blob[1], w->tau_cap);
        ts.capacity = w->tau_cap;
        ts.next_id = 1;
        if (cudaMemcpy(w->tS, &ts, sizeof(ts), cudaMemcpyHostToDevice) != cudaSuccess) {
            agb_world_destroy(w); return AGB_CUDA_ERROR;
        }
    }
    cudaMemset(w->flash_accum, 0, 8 * 4);                 // zeroed once (src/sim/step.cu:58-64)
    if (c.irr_marks) cudaMemset(c.irr_marks, 2, (size_t)w->irr_mark_bytes);   // first sweep: every line
    if (c.irr_stamp_bits) cudaMemset(c.irr_stamp_bits, 0, 4 * (size_t)w->irr_bit_words);
    cudaMemset(h.ranges, 0, 8 * (size_t)h.buckets);
    cudaMemset(h.occ, 0, 4 * (((size_t)h.buckets + 31) / 32 + 1));
    cudaMemset(h.keys_sorted, 0, 4 * n);
    cudaMemset(w->blob[0], 0, w->blob_bytes);
    cudaMemset(w->blob[1], 0, w->blob_bytes);
    cudaMemset(w->life.co2_demand, 0, 8 * (size_t)co2n);
    cudaMemset(w->life.tile_sums, 0, 4 * (size_t)stiles);       // single-pass scan status words
    cudaMemset(w->stamp_idx, 0xFF, 4 * n);
    if (cudaHostAlloc(reinterpret_cast<void**>(&w->xfer_host), 2 * sizeof(int64_t), cudaHostAllocMapped) !=
        cudaSuccess)
        w->xfer_host = nullptr;                           // export then takes the copy path
    DevState st{};
    st.cur = carve(w->blob[0], cap);
    st.spare = carve(w->blob[1], cap);
    st.next_id = 1;                                       // src/sim/cell_store.cuh:42
    if (cudaMemcpy(w->S, &st, sizeof(st), cudaMemcpyHostToDevice) != cudaSuccess) {
        agb_world_destroy(w); return AGB_CUDA_ERROR;
    }
    const agb_status ps = compute_tick_params(w);
    if (ps != AGB_OK) { agb_world_destroy(w); return ps; }
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { agb_world_destroy(w); return AGB_CUDA_ERROR; }
    *out = w;
    return AGB_OK;
}

agb_status agb_world_spawn_seeded(agb_world* w, const agb_spawn* p, uint64_t seed, agb_stream s) {
    if (!w || !p) return AGB_INVALID_ARGUMENT;
    if (p->count <= 0) return AGB_OK;
    if (p->placement == AGB_PLACE_CLUSTERS && p->clusters <= 0) return fail(w, AGB_INVALID_ARGUMENT, "clusters");
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    if (st.count + p->count > w->c.capacity) return fail(w, AGB_CAPACITY_EXCEEDED, "spawn exceeds capacity");
    Ctx c = w->c;
    c.seed = seed;
    launch_spawn(w->S, c, *p, w->blocks, s);
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

agb_status agb_world_spawn(agb_world* w, const agb_spawn* p, agb_stream s) {
    if (!w) return AGB_INVALID_ARGUMENT;
    return agb_world_spawn_seeded(w, p, w->c.seed, s);
}

agb_status agb_world_set_charge(agb_world* w, double charge, agb_stream s) {
    if (!w) return AGB_INVALID_ARGUMENT;
    // clamp01: NaN falls through both tests, as it does in the reference.
    const double q = charge < 0.0 ? 0.0 : (charge > 1.0 ? 1.0 : charge);
    if (s == nullptr && w->own_stream) s = w->own_stream;
    launch_set_charge(w->S, q * AGB_CELL_ENERGY_MAX, w->blocks, s);
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

agb_status agb_world_count(agb_world* w, int32_t* count, agb_stream s) {
    DevState st;
    const agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    *count = st.count;
    return AGB_OK;
}

agb_status agb_world_device_cells(agb_world* w, agb_cells* dev) {
    DevState st;
    const agb_status rc = read_state(w, st, nullptr);
    if (rc) return rc;
    const SoA& v = st.cur;
    agb_cells c = {v.id, v.flags, v.death_cause, v.x, v.y, v.z, v.vx, v.vy, v.vz, v.energy,
                   v.temp_cell, v.emit_power, v.dir_x, v.dir_y, v.dir_z, v.biomass, v.co2_held,
                   v.age_s, v.rng_state, v.taxis_memory, v.run_timer, v.t_local, v.irradiance,
                   v.co2_local, v.n2_local, st.count, w->c.capacity};
    *dev = c;
    return AGB_OK;
}

agb_status agb_world_import_cells(agb_world* w, const agb_cells* src, int32_t count, uint64_t next_id,
                                  agb_stream s) {
    if (!w || !src || count < 0) return AGB_INVALID_ARGUMENT;
    if (count > w->c.capacity) return fail(w, AGB_CAPACITY_EXCEEDED, "import exceeds capacity");
    void* hst[25];
    host_arrays(src, hst);
    if (host_cells_direct(w, hst)) {
        // One gather kernel; the stream's later work sees the cells. The host
        // arrays must stay valid until the stream reaches it (NULL stream: on return).
        HostCells h;
        for (int k = 0; k < 25; ++k) h.p[k] = hst[k];
        cells_import_kernel<<<xfer_blocks(count), kXferThreads, 0, s>>>(w->S, h, count, next_id);
        AGB_CUDA(w, cudaGetLastError());
        if (s == nullptr) AGB_CUDA(w, cudaStreamSynchronize(s));
        return AGB_OK;
    }
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    void* dst[25];
    soa_arrays(st.cur, dst);
    for (int k = 0; k < 25; ++k)
        if (hst[k] && count > 0)
            AGB_CUDA(w, cudaMemcpyAsync(dst[k], hst[k], kElem[k] * (size_t)count, cudaMemcpyHostToDevice, s));
    st.count = count;
    st.next_id = next_id;
    AGB_CUDA(w, cudaMemcpyAsync(&w->S->count, &st.count, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    AGB_CUDA(w, cudaMemcpyAsync(&w->S->next_id, &st.next_id, sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

agb_status agb_world_export_cells(agb_world* w, agb_cells* dst, int32_t max_count, int32_t* count,
                                  uint64_t* next_id, agb_stream s) {
    if (!w || !dst) return AGB_INVALID_ARGUMENT;
    void* hst[25];
    host_arrays(dst, hst);
    if (max_count < 0) max_count = 0;
    if (w->xfer_host && host_cells_direct(w, hst)) {
        // One scatter kernel writes the arrays and the count; one synchronisation.
        HostCells h;
        for (int k = 0; k < 25; ++k) h.p[k] = hst[k];
        const int64_t cap = max_count < w->c.capacity ? max_count : w->c.capacity;
        cells_export_kernel<<<xfer_blocks(cap), kXferThreads, 0, s>>>(w->S, h, max_count, w->xfer_host);
        AGB_CUDA(w, cudaGetLastError());
        AGB_CUDA(w, cudaStreamSynchronize(s));
        if (count) *count = (int32_t)w->xfer_host[0];
        if (next_id) *next_id = (uint64_t)w->xfer_host[1];
        dst->count = (int32_t)w->xfer_host[0];
        dst->capacity = max_count;
        return AGB_OK;
    }
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    const int32_t n = st.count < max_count ? st.count : max_count;
    void* srcp[25];
    soa_arrays(st.cur, srcp);
    for (int k = 0; k < 25; ++k)
        if (hst[k] && n > 0)
            AGB_CUDA(w, cudaMemcpyAsync(hst[k], srcp[k], kElem[k] * (size_t)n, cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    if (count) *count = st.count;
    if (next_id) *next_id = st.next_id;
    dst->count = st.count;
    dst->capacity = max_count;
    return AGB_OK;
}

agb_status agb_world_step_host(agb_world* w, const agb_cells* in, int32_t count, uint64_t next_id,
                               int32_t ticks, agb_cells* out, int32_t max_out, int32_t* out_count,
                               uint64_t* out_next_id, agb_stream s) {
    if (!w || !in || !out || ticks < 0) return AGB_INVALID_ARGUMENT;
    if (s == nullptr && ticks > 0 && !w->sg) {
        // The tick graph needs a capture-capable stream; run all three on it.
        if (!w->own_stream) AGB_CUDA(w, cudaStreamCreate(&w->own_stream));
        s = w->own_stream;
    }
    agb_status rc = agb_world_import_cells(w, in, count, next_id, s);
    if (rc != AGB_OK) return rc;
    if (ticks > 0) {
        rc = agb_world_step_graph(w, ticks, s);
        if (rc != AGB_OK) return rc;
    }
    return agb_world_export_cells(w, out, max_out, out_count, out_next_id, s);
}

agb_status agb_world_import_field(agb_world* w, int32_t f, const float* src, agb_stream s) {
    if (!w || f < 0 || f >= AGB_FIELD_COUNT || !w->c.g[f].enabled || !src) return AGB_INVALID_ARGUMENT;
    AGB_CUDA(w, cudaMemcpyAsync(field_value(w, f), src, sizeof(float) * w->c.g[f].count,
                                cudaMemcpyHostToDevice, s));
    if (f == AGB_FIELD_IRRADIANCE) irr_all_lines(w, s);
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

agb_status agb_world_export_field(agb_world* w, int32_t f, float* dst, agb_stream s) {
    if (!w || f < 0 || f >= AGB_FIELD_COUNT || !w->c.g[f].enabled || !dst) return AGB_INVALID_ARGUMENT;
    AGB_CUDA(w, cudaMemcpyAsync(dst, field_value(w, f), sizeof(float) * w->c.g[f].count,
                                cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

agb_status agb_world_export_deposit(agb_world* w, int32_t f, uint64_t* dst, agb_stream s) {
    if (!w || f < 0 || f >= AGB_FIELD_COUNT || !w->c.g[f].enabled || !dst) return AGB_INVALID_ARGUMENT;
    AGB_CUDA(w, cudaMemcpyAsync(dst, w->gdep[f], 8 * w->c.g[f].count, cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

// ---------------------------------------------------------------------------
// The predator store (taumoeba_spawn and the taumoeba_download_* readers,
// src/sim/predation.cu:420-574)
// ---------------------------------------------------------------------------
namespace {
agb_status read_tau(agb_world* w, TauState& ts, cudaStream_t s) {
    AGB_CUDA(w, cudaMemcpyAsync(&ts, w->tS, sizeof(ts), cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}
// The host arrays of agb_taumoeba with their element sizes, in TauSoA order.
void tau_host_arrays(const agb_taumoeba* a, void* out[20]) {
    void* p[20] = {a->id, a->flags, a->x, a->y, a->z, a->vx, a->vy, a->vz, a->dir_x, a->dir_y, a->dir_z,
                   a->biomass, a->prey_biomass, a->digest_timer, a->tolerance, a->generation, a->rng_state,
                   a->density_ema, a->run_timer, a->target};
    for (int k = 0; k < 20; ++k) out[k] = p[k];
}
void tau_dev_arrays(const TauSoA& t, void* out[20]) {
    void* p[20] = {t.id, t.flags, t.x, t.y, t.z, t.vx, t.vy, t.vz, t.dir_x, t.dir_y, t.dir_z, t.biomass,
                   t.prey_biomass, t.digest_timer, t.tolerance, t.generation, t.rng_state, t.density_ema,
                   t.run_timer, t.target};
    for (int k = 0; k < 20; ++k) out[k] = p[k];
}
const size_t TAU_WIDTH[20] = {8, 4, 8, 8, 8, 8, 8, 8, 4, 4, 4, 8, 8, 4, 4, 4, 8, 4, 4, 4};
void set_tau_active(agb_world* w) {
    if (!w->tau_active) {
        w->tau_active = true;
        invalidate_graphs(w);                             // captured ticks lack the predation stage
    }
}
}  // namespace

agb_status agb_world_spawn_taumoeba(agb_world* w, int32_t count, uint64_t seed, agb_stream s) {
    if (!w || count < 0) return AGB_INVALID_ARGUMENT;
    if (count == 0) return AGB_OK;
    TauState ts;
    agb_status rc = read_tau(w, ts, s);
    if (rc) return rc;
    if (ts.count + count > ts.capacity) return fail(w, AGB_CAPACITY_EXCEEDED, "taumoeba spawn exceeds capacity");
    launch_tau_spawn(w->tS, count, seed, w->taup, s);
    AGB_CUDA(w, cudaGetLastError());
    set_tau_active(w);
    return AGB_OK;
}

agb_status agb_world_import_taumoeba(agb_world* w, const agb_taumoeba* src, int32_t count, uint64_t next_id,
                                     agb_stream s) {
    if (!w || !src || count < 0) return AGB_INVALID_ARGUMENT;
    if (count > w->tau_cap) return fail(w, AGB_CAPACITY_EXCEEDED, "taumoeba import exceeds capacity");
    TauState ts;
    agb_status rc = read_tau(w, ts, s);
    if (rc) return rc;
    void* h[20];
    void* d[20];
    tau_host_arrays(src, h);
    tau_dev_arrays(ts.cur, d);
    for (int k = 0; k < 20; ++k) {
        if (!h[k]) return AGB_INVALID_ARGUMENT;
        if (count > 0) AGB_CUDA(w, cudaMemcpyAsync(d[k], h[k], TAU_WIDTH[k] * (size_t)count, cudaMemcpyHostToDevice, s));
    }
    ts.count = count;
    ts.next_id = next_id;
    AGB_CUDA(w, cudaMemcpyAsync(w->tS, &ts, sizeof(ts), cudaMemcpyHostToDevice, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    if (count > 0) set_tau_active(w);
    return AGB_OK;
}

agb_status agb_world_export_taumoeba(agb_world* w, agb_taumoeba* dst, int32_t max_count, int32_t* count,
                                     uint64_t* next_id, agb_stream s) {
    if (!w || !dst || max_count < 0) return AGB_INVALID_ARGUMENT;
    TauState ts;
    agb_status rc = read_tau(w, ts, s);
    if (rc) return rc;
    const int32_t n = ts.count < max_count ? ts.count : max_count;
    void* h[20];
    void* d[20];
    tau_host_arrays(dst, h);
    tau_dev_arrays(ts.cur, d);
    for (int k = 0; k < 20; ++k)
        if (h[k] && n > 0) AGB_CUDA(w, cudaMemcpyAsync(h[k], d[k], TAU_WIDTH[k] * (size_t)n, cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    if (count) *count = ts.count;
    if (next_id) *next_id = ts.next_id;
    return AGB_OK;
}

agb_status agb_world_set_flash(agb_world* w, int32_t active, double power) {
    if (!w || !std::isfinite(power)) return AGB_INVALID_ARGUMENT;
    const bool on = active != 0;
    const double pw = power > 0.0 ? power : AGB_PETROVA_FLASH_POWER;
    if (on != w->flash_active || pw != w->flash_power) {
        w->flash_active = on;
        w->flash_power = pw;
        invalidate_graphs(w);                             // captured ticks baked the old stage
    }
    return AGB_OK;
}

agb_status agb_world_flash_audit(agb_world* w, double* impulse_ns, double* discharged_j) {
    if (!w || !impulse_ns || !discharged_j) return AGB_INVALID_ARGUMENT;
    unsigned long long raw[4];
    AGB_CUDA(w, cudaDeviceSynchronize());
    AGB_CUDA(w, cudaMemcpy(raw, w->flash_accum, sizeof(raw), cudaMemcpyDeviceToHost));
    const double ix = (double)(long long)raw[0] / AGB_FLASH_IMPULSE_SCALE;
    const double iy = (double)(long long)raw[1] / AGB_FLASH_IMPULSE_SCALE;
    const double iz = (double)(long long)raw[2] / AGB_FLASH_IMPULSE_SCALE;
    *impulse_ns = std::sqrt(ix * ix + iy * iy + iz * iz);
    *discharged_j = (double)(long long)raw[3] / AGB_FLASH_ENERGY_SCALE;
    return AGB_OK;
}

agb_status agb_world_apply_brush(agb_world* w, int32_t kind, double x, double y, double radius,
                                 double strength, agb_stream s) {
    if (!w) return AGB_INVALID_ARGUMENT;
    int32_t f;
    double amount = strength;
    switch (kind) {
        case AGB_BRUSH_HEAT: f = AGB_FIELD_TEMPERATURE; break;
        case AGB_BRUSH_CHILL: f = AGB_FIELD_TEMPERATURE; amount = -strength; break;
        case AGB_BRUSH_INJECT_CO2: f = AGB_FIELD_CO2; break;
        case AGB_BRUSH_INJECT_N2: f = AGB_FIELD_N2; break;
        default: return fail(w, AGB_INVALID_ARGUMENT, "unknown brush");
    }
    if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite(radius) || !std::isfinite(strength))
        return fail(w, AGB_INVALID_ARGUMENT, "brush arguments must be finite");
    const GridDev& g = w->c.g[f];
    if (!g.enabled) return fail(w, AGB_INVALID_ARGUMENT, "brush on a field the world does not have");
    if (radius <= 0.0) return AGB_OK;                  // grid_brush: an empty brush is a no-op
    const float cx = (float)x, cy = (float)y, rad = (float)radius;
    // Columns whose centres can lie within the disc, with two voxels of margin
    // for float rounding; the kernel applies the exact test to each.
    auto span = [&](float c, float half, int32_t n, int32_t& lo, int32_t& cnt) {
        const double a = std::floor(((double)c - rad + half) / g.dxf - 0.5) - 2.0;
        const double b = std::ceil(((double)c + rad + half) / g.dxf - 0.5) + 2.0;
        const double l = a < 0.0 ? 0.0 : a, h = b > n - 1.0 ? n - 1.0 : b;
        lo = (int32_t)l;
        cnt = h >= l ? (int32_t)(h - l) + 1 : 0;
    };
    int32_t x0, bw, y0, bh;
    span(cx, g.hx, g.nx, x0, bw);
    span(cy, g.hy, g.ny, y0, bh);
    if (s == nullptr && w->own_stream) s = w->own_stream;
    launch_brush(field_value(w, f), g, cx, cy, rad, (float)amount, x0, y0, bw, bh, s);
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

agb_status agb_world_step(agb_world* w, int32_t ticks, agb_stream s) {
    if (!w || ticks < 0) return AGB_INVALID_ARGUMENT;
    for (int32_t t = 0; t < ticks; ++t) tick_once(w, s);
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

// Captures `ticks` ticks from the world's current host-side state into a new
// cached graph (not launched). Capture runs tick_once, which advances the
// host-side tick state (buffer parities, tick, clock) as the replay will.
static agb_status capture_entry(agb_world* w, int32_t ticks, cudaStream_t s, GraphEntry** out) {
    const uint64_t P = w->d.compaction_period > 0 ? (uint64_t)w->d.compaction_period : 1;
    cudaGraph_t graph;
    GraphEntry e{ticks, parity_bits(w), w->tick % P, nullptr, 0, 0};
    AGB_CUDA(w, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int32_t t = 0; t < ticks; ++t) tick_once(w, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) return cuda_fail(w, ce, "cudaStreamEndCapture");
    e.parity_after = parity_bits(w);
    {
        size_t nn = 0;
        cudaGraphGetNodes(graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++e.kernels;
        }
    }
    const cudaError_t ie = cudaGraphInstantiate(&e.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_fail(w, ie, "cudaGraphInstantiate");
    w->graphs.push_back(e);
    *out = &w->graphs.back();
    return AGB_OK;
}

static GraphEntry* find_entry(agb_world* w, int32_t ticks) {
    const uint64_t P = w->d.compaction_period > 0 ? (uint64_t)w->d.compaction_period : 1;
    const uint32_t par = parity_bits(w);
    const uint64_t phase = w->tick % P;
    for (GraphEntry& g : w->graphs)
        if (g.ticks == ticks && g.parity == par && g.tick_phase == phase) return &g;
    return nullptr;
}

// The host-side effect of replaying a cached graph: buffer parities, tick, clock.
static void advance_as_replay(agb_world* w, const GraphEntry& g) {
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) w->gcur[f] = (g.parity_after >> f) & 1;
    refresh_grid_ptrs(w);
    w->tick += (uint64_t)g.ticks;
    w->sim_time += w->tp.dt * g.ticks;
}

agb_status agb_world_step_graph(agb_world* w, int32_t ticks, agb_stream s) {
    if (!w || ticks <= 0) return AGB_INVALID_ARGUMENT;
    if (w->sg) return agb_world_step(w, ticks, s);    // the judge reads results on the host: no capture
    if (s == nullptr && w->own_stream) s = w->own_stream;
    if (GraphEntry* g = find_entry(w, ticks)) {
        AGB_CUDA(w, cudaGraphLaunch(g->exec, s));
        w->graph_kernels_total += g->kernels;
        advance_as_replay(w, *g);
        return AGB_OK;
    }
    if (s == nullptr) {
        // Capture needs a stream other than the legacy default one; a blocking
        // stream keeps the launch ordered with the caller's default-stream work.
        if (!w->own_stream) AGB_CUDA(w, cudaStreamCreate(&w->own_stream));
        s = w->own_stream;
    }
    GraphEntry* g = nullptr;
    const agb_status rc = capture_entry(w, ticks, s, &g);
    if (rc != AGB_OK) return rc;
    w->graph_kernels_total += g->kernels;
    // Capture advanced the host-side tick state; the graph has not run yet.
    AGB_CUDA(w, cudaGraphLaunch(g->exec, s));
    return AGB_OK;
}

agb_status agb_world_prepare_graphs(agb_world* w, int32_t ticks, agb_stream stream) {
    if (!w || ticks <= 0) return AGB_INVALID_ARGUMENT;
    if (w->sg) return AGB_OK;                           // surrogate-driven worlds step eagerly
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (s == nullptr) {
        if (!w->own_stream) AGB_CUDA(w, cudaStreamCreate(&w->own_stream));
        s = w->own_stream;
    }
    int saved_gcur[AGB_FIELD_COUNT];
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) saved_gcur[f] = w->gcur[f];
    const uint64_t saved_tick = w->tick;
    const double saved_time = w->sim_time;
    // Walk the (buffer parities, tick phase) states that stepping by `ticks`
    // visits from here until one repeats; capture each state's graph once.
    const uint64_t P = w->d.compaction_period > 0 ? (uint64_t)w->d.compaction_period : 1;
    const uint64_t limit = 4 * P * (uint64_t)(1u << AGB_FIELD_COUNT) + 8;
    std::vector<std::pair<uint32_t, uint64_t>> seen;
    agb_status rc = AGB_OK;
    for (uint64_t it = 0; it < limit && rc == AGB_OK; ++it) {
        const std::pair<uint32_t, uint64_t> key{parity_bits(w), w->tick % P};
        bool repeat = false;
        for (const auto& k : seen) repeat = repeat || (k == key);
        if (repeat) break;
        seen.push_back(key);
        if (GraphEntry* g = find_entry(w, ticks)) {
            advance_as_replay(w, *g);
        } else {
            GraphEntry* ng = nullptr;
            rc = capture_entry(w, ticks, s, &ng);
        }
    }
    for (int f = 0; f < AGB_FIELD_COUNT; ++f) w->gcur[f] = saved_gcur[f];
    refresh_grid_ptrs(w);
    w->tick = saved_tick;
    w->sim_time = saved_time;
    return rc;
}

agb_status agb_world_set_timing(agb_world* w, int32_t enable) {
    if (!w) return AGB_INVALID_ARGUMENT;
    const bool on = enable != 0;
    if (on && !w->tev[0])
        for (cudaEvent_t& e : w->tev) AGB_CUDA(w, cudaEventCreate(&e));
    if (on != w->timing) {
        w->timing = on;
        invalidate_graphs(w);
    }
    return AGB_OK;
}

agb_status agb_world_section_times(agb_world* w, float ms[AGB_TICK_SECTIONS]) {
    if (!w || !ms) return AGB_INVALID_ARGUMENT;
    for (int k = 0; k < AGB_TICK_SECTIONS; ++k) ms[k] = -1.0f;
    if (!w->timing) return AGB_OK;
    AGB_CUDA(w, cudaEventSynchronize(w->tev[2 * AGB_SECTION_TICK + 1]));
    for (int k = 0; k < AGB_TICK_SECTIONS; ++k) {
        float t = -1.0f;
        if (cudaEventElapsedTime(&t, w->tev[2 * k], w->tev[2 * k + 1]) != cudaSuccess) t = -1.0f;
        ms[k] = t;
    }
    (void)cudaGetLastError();     // a section that has not run leaves an unrecorded event: not an error here
    return AGB_OK;
}

agb_status agb_world_attach_surrogate(agb_world* w, agb_surrogate* sg, agb_stream stream) {
    if (!w) return AGB_INVALID_ARGUMENT;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const GridDev& T = w->c.g[AGB_FIELD_TEMPERATURE];
    const GridDev& C = w->c.g[AGB_FIELD_CO2];
    if (!sg) {
        if (w->sg && w->sg_q) {
            // Detaching mid-window: fold the heat accumulated so far into the grid.
            surrogate_source_from_deposit(w->gdep[AGB_FIELD_TEMPERATURE], w->sg_q, T.count, 1.0 / T.scale, 1, s);
            surrogate_add(field_value(w, AGB_FIELD_TEMPERATURE), w->sg_q, T.count, s);
        }
        w->sg = nullptr;
        invalidate_graphs(w);
        AGB_CUDA(w, cudaGetLastError());
        return AGB_OK;
    }
    int32_t dims[3], steps = 0, bc[2][6];
    float coeff[2];
    surrogate_info(sg, dims, &steps, coeff, bc);
    if (!T.enabled || !C.enabled || T.nx != dims[0] || T.ny != dims[1] || T.nz != dims[2] || C.nx != dims[0] ||
        C.ny != dims[1] || C.nz != dims[2])
        return fail(w, AGB_INVALID_ARGUMENT, "surrogate grid differs from the world's temperature/CO2 grids");
    if (w->tp.t_substeps != 1 || w->tp.c_substeps != 1 || coeff[0] != w->tp.t_coeff || coeff[1] != w->tp.c_coeff)
        return fail(w, AGB_INVALID_ARGUMENT, "surrogate FTCS step differs from the world's (one pass per tick)");
    for (int k = 0; k < 6; ++k)
        if (bc[0][k] != w->gbc[AGB_FIELD_TEMPERATURE][k] || bc[1][k] != w->gbc[AGB_FIELD_CO2][k])
            return fail(w, AGB_INVALID_ARGUMENT, "surrogate boundary conditions differ from the world's");
    if (!w->sg_q && dalloc(w, &w->sg_q, 4 * (size_t)T.count) != cudaSuccess) return AGB_OUT_OF_MEMORY;
    w->sg = sg;
    w->sg_steps = steps;
    invalidate_graphs(w);
    return AGB_OK;
}

agb_status agb_world_set_walk(agb_world* w, int32_t lanes, int32_t fused) {
    if (!w || (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8) || (fused != 0 && fused != 1))
        return AGB_INVALID_ARGUMENT;
    if (w->walk_lanes != lanes || w->fuse_cells != (fused != 0)) {
        w->walk_lanes = lanes;
        w->fuse_cells = fused != 0;
        invalidate_graphs(w);
    }
    return AGB_OK;
}

agb_status agb_world_walk(agb_world* w, int32_t* lanes, int32_t* fused) {
    if (!w || !lanes || !fused) return AGB_INVALID_ARGUMENT;
    *lanes = w->walk_lanes;
    *fused = w->fuse_cells ? 1 : 0;
    return AGB_OK;
}

agb_status agb_world_graph_kernels(agb_world* w, int64_t* kernels) {
    if (!w || !kernels) return AGB_INVALID_ARGUMENT;
    *kernels = w->graph_kernels_total;
    return AGB_OK;
}

agb_status agb_world_stage(agb_world* w, int32_t stage, agb_stream s) {
    if (!w) return AGB_INVALID_ARGUMENT;
    switch (stage) {
        case AGB_STAGE_HASH: stage_hash(w, s); break;
        case AGB_STAGE_THERMAL: stage_thermal(w, s); break;
        case AGB_STAGE_EMISSION: stage_emission(w, s); break;
        case AGB_STAGE_TAXIS: launch_taxis(w->S, w->c, w->tp, w->blocks, s); break;
        case AGB_STAGE_FLASH:
            if (w->flash_active) launch_flash(w->S, w->tp.dt, w->flash_power, w->flash_accum, w->blocks, s);
            break;
        case AGB_STAGE_PREDATION: stage_predation(w, s); break;
        case AGB_STAGE_MOTION: stage_motion(w, s); break;
        case AGB_STAGE_SLOW_FIELDS: stage_slow_fields(w, s); break;
        case AGB_STAGE_LIFECYCLE: stage_lifecycle(w, s); break;
        case AGB_STAGE_COMPACT: launch_compact(w->S, w->c, w->life, w->blocks, s); break;
        case AGB_STAGE_CLOCK: stage_clock(w); break;
        default: return AGB_INVALID_ARGUMENT;
    }
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

agb_status agb_world_diffuse(agb_world* w, int32_t f, double dt, agb_stream s) {
    if (!w || f < 0 || f >= AGB_FIELD_COUNT) return AGB_INVALID_ARGUMENT;
    const GridDev& g = w->c.g[f];
    if (!g.enabled) return AGB_OK;
    if (f == AGB_FIELD_IRRADIANCE) irr_all_lines(w, s);
    const double D = w->d.grid[f].diffusivity;
    const int32_t steps = substeps_for(g, D, dt);         // grid_diffuse, diffuse.cu:159-186
    if (steps <= 0) return AGB_OK;
    const float coeff = (float)(D * (dt / steps) / (g.dx * g.dx));
    if (!coeff_ok(g, coeff)) return fail(w, AGB_INVALID_ARGUMENT, "diffusion coefficient unstable");
    for (int32_t k = 0; k < steps; ++k) ftcs(w, f, coeff, s);
    AGB_CUDA(w, cudaGetLastError());
    return AGB_OK;
}

agb_status agb_world_stats(agb_world* w, agb_stats* out, agb_stream s) {
    if (!w || !out) return AGB_INVALID_ARGUMENT;
    refresh_grid_ptrs(w);
    launch_stats(w->S, w->c, w->acc, w->blocks, s);
    if (w->tau_active) launch_tau_stats(w->tS, w->tau_cap, w->acc, s);
    AGB_CUDA(w, cudaGetLastError());
    AGB_CUDA(w, cudaMemcpyAsync(w->acc_host, w->acc, sizeof(w->acc_host), cudaMemcpyDeviceToHost, s));
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    const unsigned long long* a = w->acc_host;
    auto fx = [](unsigned long long raw, double scale) { return (double)(long long)raw / scale; };
    agb_stats r;
    std::memset(&r, 0, sizeof(r));
    r.tick = w->tick;                                     // world_stats, src/sim/stats.cu:102-153
    r.sim_time_s = w->sim_time;
    r.physics_rate = w->physics_rate;
    r.biology_rate = w->biology_rate;
    const unsigned n_alive = (unsigned)a[7], n_dead = (unsigned)a[8];
    r.n_live = (int32_t)n_alive;
    r.n_dead = (int32_t)n_dead;
    r.n_awake = (int32_t)a[9];
    r.n_dormant = (int32_t)a[10];
    r.total_energy_j = fx(a[0], AGB_DEPOSIT_SCALE_STATS);
    r.mean_charge = (n_alive + n_dead) > 0u ? r.total_energy_j / ((n_alive + n_dead) * AGB_CELL_ENERGY_MAX) : 0.0;
    r.mean_temp_cell_k = n_alive > 0u ? fx(a[1], AGB_DEPOSIT_SCALE_STATS) / n_alive : 0.0;
    const GridDev& T = w->c.g[AGB_FIELD_TEMPERATURE];
    const double cells = T.enabled ? (double)T.count : 0.0;
    r.mean_temp_medium_k = cells > 0.0 ? fx(a[2], AGB_DEPOSIT_SCALE_STATS) / cells : 0.0;
    r.max_temp_medium_k = fx(a[5], AGB_DEPOSIT_SCALE_STATS);
    const GridDev& C2 = w->c.g[AGB_FIELD_CO2];
    const GridDev& N2 = w->c.g[AGB_FIELD_N2];
    const double vc = C2.enabled ? C2.dx * C2.dx * C2.dz_eff : 0.0;
    const double vn = N2.enabled ? N2.dx * N2.dx * N2.dz_eff : 0.0;
    r.co2_total_kg = fx(a[3], AGB_STATS_SCALE_FIELD) * vc;
    r.n2_total_kg = fx(a[4], AGB_STATS_SCALE_FIELD) * vn;
    r.divisions_this_window = st.divisions_this_window;
    r.deaths_this_window = (int32_t)(st.deaths_total - w->deaths_reported);
    w->deaths_reported = st.deaths_total;
    const int32_t zero = 0;
    AGB_CUDA(w, cudaMemcpyAsync(&w->S->divisions_this_window, &zero, sizeof(zero), cudaMemcpyHostToDevice, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    r.boil_events = r.max_temp_medium_k >= AGB_WATER_BOILING_POINT ? 1 : 0;
    r.n_taumoeba = (int32_t)a[11];
    r.mean_tau_tolerance = a[11] > 0u ? fx(a[6], AGB_DEPOSIT_SCALE_STATS) / (double)a[11] : 0.0;
    *out = r;
    return AGB_OK;
}

agb_status agb_world_stats_accum(agb_world* w, uint64_t out[12]) {
    if (!w || !out) return AGB_INVALID_ARGUMENT;
    for (int k = 0; k < 12; ++k) out[k] = w->acc_host[k];
    return AGB_OK;
}

agb_status agb_world_set_clock(agb_world* w, double p, double b) {   // world_set_clock, step.cu:206-215
    if (!w) return AGB_INVALID_ARGUMENT;
    w->physics_rate = p < AGB_CLOCK_PHYSICS_MIN ? AGB_CLOCK_PHYSICS_MIN : (p > AGB_CLOCK_PHYSICS_MAX ? AGB_CLOCK_PHYSICS_MAX : p);
    w->biology_rate = b < AGB_CLOCK_BIOLOGY_MIN ? AGB_CLOCK_BIOLOGY_MIN : (b > AGB_CLOCK_BIOLOGY_MAX ? AGB_CLOCK_BIOLOGY_MAX : b);
    invalidate_graphs(w);
    return compute_tick_params(w);
}

agb_status agb_world_set_rates(agb_world* w, double p, double b) {
    if (!w) return AGB_INVALID_ARGUMENT;
    if (!(std::isfinite(p) && p > 0.0 && std::isfinite(b) && b > 0.0))
        return fail(w, AGB_INVALID_ARGUMENT, "clock rates must be finite and positive");
    w->physics_rate = p;
    w->biology_rate = b;
    invalidate_graphs(w);
    return compute_tick_params(w);
}

agb_status agb_world_set_overrides(agb_world* w, double co2_mass_per_division, double max_emit_power) {
    if (!w) return AGB_INVALID_ARGUMENT;
    if (!std::isfinite(co2_mass_per_division) || !std::isfinite(max_emit_power))
        return fail(w, AGB_INVALID_ARGUMENT, "overrides must be finite");
    w->d.co2_mass_per_division = co2_mass_per_division;
    w->d.max_emit_power = max_emit_power;
    w->c.co2_quota = co2_mass_per_division;
    invalidate_graphs(w);
    return compute_tick_params(w);
}

agb_status agb_world_set_light(agb_world* w, const agb_light* light) {
    if (!w || !light) return AGB_INVALID_ARGUMENT;
    w->d.light = *light;
    compute_light(w);
    invalidate_graphs(w);
    // Every line's unshadowed value (and the line numbering) may change: the
    // next sweep rewrites them all.
    AGB_CUDA(w, cudaDeviceSynchronize());
    irr_all_lines(w, nullptr);
    AGB_CUDA(w, cudaDeviceSynchronize());
    return AGB_OK;
}

agb_status agb_world_set_boundary(agb_world* w, int32_t field, const int32_t bc[6], const double face_value[6]) {
    if (!w || !bc || !face_value || field < 0 || field >= AGB_FIELD_COUNT) return AGB_INVALID_ARGUMENT;
    if (!w->c.g[field].enabled) return fail(w, AGB_INVALID_ARGUMENT, "boundary of a field the world does not have");
    for (int k = 0; k < 6; ++k) {
        if (bc[k] < AGB_BC_DIRICHLET || bc[k] > AGB_BC_ROBIN) return fail(w, AGB_INVALID_ARGUMENT, "boundary kind");
        if (!std::isfinite(face_value[k])) return fail(w, AGB_INVALID_ARGUMENT, "face value must be finite");
    }
    for (int k = 0; k < 6; ++k) {
        w->d.grid[field].bc[k] = bc[k];
        w->d.grid[field].face_value[k] = face_value[k];
        w->gbc[field][k] = bc[k];
        w->gface[field][k] = (float)face_value[k];
    }
    invalidate_graphs(w);                              // captured passes baked the old faces
    return AGB_OK;
}

agb_status agb_world_export_hash(agb_world* w, int32_t dims[4], uint32_t* keys_sorted, uint32_t* vals_sorted,
                                 int32_t* bucket_start, int32_t* bucket_end, agb_stream s) {
    if (!w || !dims) return AGB_INVALID_ARGUMENT;
    const HashDev& h = w->c.h;
    dims[0] = h.nx; dims[1] = h.ny; dims[2] = h.nz; dims[3] = h.buckets;
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    const int32_t n = st.hash_count;
    if (keys_sorted && n > 0)
        AGB_CUDA(w, cudaMemcpyAsync(keys_sorted, h.keys_sorted, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (vals_sorted && n > 0)
        AGB_CUDA(w, cudaMemcpyAsync(vals_sorted, h.vals_sorted, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (bucket_start || bucket_end) {
        std::vector<int2> r((size_t)h.buckets);
        AGB_CUDA(w, cudaMemcpyAsync(r.data(), h.ranges, 8 * (size_t)h.buckets, cudaMemcpyDeviceToHost, s));
        AGB_CUDA(w, cudaStreamSynchronize(s));
        for (int32_t b = 0; b < h.buckets; ++b) {
            if (bucket_start) bucket_start[b] = r[b].x;
            if (bucket_end) bucket_end[b] = r[b].y;
        }
    }
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

agb_status agb_world_export_forces(agb_world* w, float* fx, float* fy, float* fz, agb_stream s) {
    if (!w) return AGB_INVALID_ARGUMENT;
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    const size_t b = 4 * (size_t)st.count;
    if (b) {
        if (fx) AGB_CUDA(w, cudaMemcpyAsync(fx, w->fx, b, cudaMemcpyDeviceToHost, s));
        if (fy) AGB_CUDA(w, cudaMemcpyAsync(fy, w->fy, b, cudaMemcpyDeviceToHost, s));
        if (fz) AGB_CUDA(w, cudaMemcpyAsync(fz, w->fz, b, cudaMemcpyDeviceToHost, s));
    }
    AGB_CUDA(w, cudaStreamSynchronize(s));
    return AGB_OK;
}

agb_status agb_world_mirror(agb_world* w, agb_mirror* out, agb_stream s) {
    if (!w || !out) return AGB_INVALID_ARGUMENT;
    DevState st;
    TauState ts{};
    AGB_CUDA(w, cudaMemcpyAsync(&st, w->S, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    if (w->tS) AGB_CUDA(w, cudaMemcpyAsync(&ts, w->tS, sizeof(TauState), cudaMemcpyDeviceToHost, s));
    AGB_CUDA(w, cudaStreamSynchronize(s));
    const SoA& v = st.cur;
    agb_cells c = {v.id, v.flags, v.death_cause, v.x, v.y, v.z, v.vx, v.vy, v.vz, v.energy,
                   v.temp_cell, v.emit_power, v.dir_x, v.dir_y, v.dir_z, v.biomass, v.co2_held,
                   v.age_s, v.rng_state, v.taxis_memory, v.run_timer, v.t_local, v.irradiance,
                   v.co2_local, v.n2_local, st.count, w->c.capacity};
    out->cells = c;
    out->next_id = st.next_id;
    out->divisions_this_window = st.divisions_this_window;
    out->deaths_total = st.deaths_total;
    out->dead_slots_prev = st.dead_slots_prev;
    out->error = st.error;
    out->tau_count = w->tS ? ts.count : 0;
    out->tau_next_id = w->tS ? ts.next_id : 1;
    return AGB_OK;
}

agb_status agb_world_counters(agb_world* w, int64_t out[4], agb_stream s) {
    if (!w || !out) return AGB_INVALID_ARGUMENT;
    DevState st;
    agb_status rc = read_state(w, st, s);
    if (rc) return rc;
    out[0] = st.divisions_this_window;
    out[1] = st.deaths_total;
    out[2] = st.dead_slots_prev;
    out[3] = st.error;
    return AGB_OK;
}

}  // extern "C"
