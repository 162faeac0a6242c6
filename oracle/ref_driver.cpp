// oracle/ref_driver.cpp -- C entry points over the REFERENCE's own World API
// (src/sim/world.cuh:183-243, src/fields/grid.cuh:87-103, src/sim/hash.cuh:50-53),
// compiled together with the reference's unmodified src/sim + src/fields sources
// under the host emulation in oracle/ref_emu/. Used only to generate and check
// golden fixtures in this repository's tests; it is the reference itself, run on
// the CPU, not a restatement.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>

#include "contracts/cell_store_v1.h"
#include "contracts/telemetry_v1.h"
#include "fields/grid.cuh"
#include "sim/accept.h"
#include "sim/scenario.h"
#include "sim/snapshot.h"
#include "sim/world.cuh"

#include <vector>

namespace emu {
uint3 g_block_idx{0, 0, 0}, g_thread_idx{0, 0, 0};
dim3 g_block_dim{1, 1, 1}, g_grid_dim{1, 1, 1};
static size_t g_live = 0;
size_t live_allocations() { return g_live; }
void* alloc(size_t bytes) {
    void* p = nullptr;
    if (posix_memalign(&p, 256, bytes ? bytes : 1) != 0) return nullptr;
    std::memset(p, 0, bytes);   // reference never relies on garbage; zero keeps runs reproducible
    ++g_live;
    return p;
}
void release(void* p) { if (p) { std::free(p); --g_live; } }
}  // namespace emu

using namespace astro;
using namespace astro::sim;
using astro::contract::BoundaryCondition;

extern "C" {

// Flat knob block; every field maps onto WorldDesc/MotionConfig/World members.
struct RefParams {
    double chamber_w, chamber_h, chamber_d;
    int32_t capacity;
    uint64_t seed;
    uint8_t boundary_x, boundary_y, gravity_axis, thermal_noise;
    uint8_t contact_enabled, adhesion_enabled, thermal_enabled, emission_enabled;
    uint8_t taxis_enabled, occlusion_exact, store_disposition, compaction_enabled;
    double ambient_temp, co2_init;
    int32_t n_temp, n_co2, n_n2, n_irr;       // 0 = canon resolution
    int32_t bc_temp, bc_co2;                  // -1 = reference default
    float light_dir_x, light_dir_y, light_irradiance, ambient_irradiance;
    uint8_t light_enabled;
    double physics_rate, biology_rate, co2_mass_per_division;
    int32_t tau_capacity;                     // 0 = the reference default
    uint8_t tau_compaction;
};

struct RefSpawn {
    int32_t count, placement, charge_dist, awake;
    double place_x, place_y, place_radius, charge_a, charge_b;
};

static void regrid(fields::Grid2D& g, int32_t n, double extent, int32_t bc) {
    if (n <= 0 && bc < 0) return;
    const fields::Grid2D old = g;
    const int32_t nn = n > 0 ? n : old.n;
    const BoundaryCondition b = bc >= 0 ? static_cast<BoundaryCondition>(bc) : old.bc;
    fields::grid_destroy(g);
    fields::grid_create(g, nn, extent, old.diffusivity, old.ambient, old.deposit_scale, b,
                        canon::DT_PHYSICS);
}

void* ref_world_create(const RefParams* p) {
    World* w = new (std::nothrow) World{};
    if (!w) return nullptr;
    WorldDesc d{};
    d.chamber = Chamber{p->chamber_w, p->chamber_h, p->chamber_d};
    d.capacity = p->capacity;
    d.tau_capacity = p->tau_capacity;
    d.seed = p->seed;
    MotionConfig m{};
    m.boundary_x = static_cast<Boundary>(p->boundary_x);
    m.boundary_y = static_cast<Boundary>(p->boundary_y);
    m.gravity_axis = static_cast<GravityAxis>(p->gravity_axis);
    m.thermal_noise = p->thermal_noise;
    m.contact_enabled = p->contact_enabled;
    m.adhesion_enabled = p->adhesion_enabled;
    m.thermal_enabled = p->thermal_enabled;
    m.emission_enabled = p->emission_enabled;
    m.taxis_enabled = p->taxis_enabled;
    m.occlusion_exact = p->occlusion_exact;
    m.ambient_temp = p->ambient_temp;
    m.store_disposition = static_cast<contract::StoreDisposition>(p->store_disposition);
    m.compaction_enabled = p->compaction_enabled;
    m.tau_compaction_enabled = p->tau_compaction != 0;
    d.motion = m;
    d.co2_init = p->co2_init;
    if (world_create(*w, d)) { delete w; return nullptr; }
    regrid(w->fields.temperature, p->n_temp, d.chamber.w, p->bc_temp);
    regrid(w->fields.co2, p->n_co2, d.chamber.w, p->bc_co2);
    regrid(w->fields.n2, p->n_n2, d.chamber.w, -1);
    regrid(w->fields.irradiance, p->n_irr, d.chamber.w, -1);
    w->light = contract::LightSource{p->light_dir_x, p->light_dir_y, p->light_irradiance, 0.0f,
                                     p->light_enabled};
    w->ambient_irradiance = p->ambient_irradiance;
    w->physics_rate = p->physics_rate;
    w->biology_rate = p->biology_rate;
    w->co2_mass_per_division = p->co2_mass_per_division;
    return w;
}

void ref_world_destroy(void* h) {
    World* w = static_cast<World*>(h);
    world_destroy(*w);
    delete w;
}

int ref_spawn(void* h, const RefSpawn* s) {
    World* w = static_cast<World*>(h);
    SpawnParams p{};
    p.count = s->count;
    p.placement = static_cast<Placement>(s->placement);
    p.place_x = s->place_x; p.place_y = s->place_y; p.place_radius = s->place_radius;
    p.charge_dist = static_cast<Distribution>(s->charge_dist);
    p.charge_a = s->charge_a; p.charge_b = s->charge_b;
    p.awake = s->awake != 0;
    return static_cast<int>(cell_store_spawn(w->cells, p, w->chamber, w->seed).status);
}

int32_t ref_count(void* h) { return static_cast<World*>(h)->cells.count; }
uint64_t ref_next_id(void* h) { return static_cast<World*>(h)->cells.next_id; }

// The 25 SoA arrays of contracts/cell_store_v1.h, in declaration order.
static void soa_ptrs(const contract::CellStoreView& v, void* out[25], size_t sz[25]) {
    void* p[25] = {v.id, v.flags, v.death_cause, v.x, v.y, v.z, v.vx, v.vy, v.vz, v.energy,
                   v.temp_cell, v.emit_power, v.dir_x, v.dir_y, v.dir_z, v.biomass, v.co2_held,
                   v.age_s, v.rng_state, v.taxis_memory, v.run_timer, v.t_local, v.irradiance,
                   v.co2_local, v.n2_local};
    const size_t s[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};
    for (int k = 0; k < 25; ++k) { out[k] = p[k]; sz[k] = s[k]; }
}

// dir 0: engine -> host buffers; dir 1: host buffers -> engine (sets count/next_id).
int ref_cells_io(void* h, int dir, void** host, int32_t count, uint64_t next_id) {
    World* w = static_cast<World*>(h);
    if (count < 0 || count > w->cells.capacity) return 1;
    void* dev[25]; size_t sz[25];
    soa_ptrs(w->cells.view, dev, sz);
    for (int k = 0; k < 25; ++k) {
        if (!host[k]) continue;
        if (dir == 0) std::memcpy(host[k], dev[k], sz[k] * static_cast<size_t>(count));
        else std::memcpy(dev[k], host[k], sz[k] * static_cast<size_t>(count));
    }
    if (dir == 1) {
        w->cells.count = count;
        w->cells.view.count = count;
        w->cells.next_id = next_id;
    }
    return 0;
}

static fields::Grid2D* field(World* w, int fid) {
    switch (fid) {
        case 0: return &w->fields.temperature;
        case 1: return &w->fields.co2;
        case 2: return &w->fields.n2;
        case 3: return &w->fields.irradiance;
    }
    return nullptr;
}

int32_t ref_field_n(void* h, int fid) { return field(static_cast<World*>(h), fid)->n; }

int ref_field_io(void* h, int fid, int dir, float* host) {
    fields::Grid2D* g = field(static_cast<World*>(h), fid);
    if (!g) return 1;
    const size_t bytes = sizeof(float) * static_cast<size_t>(g->n) * g->n;
    if (dir == 0) std::memcpy(host, g->value, bytes);
    else std::memcpy(g->value, host, bytes);
    return 0;
}

// Raw fixed-point accumulator of a field (the irradiance one holds occlusion).
int ref_field_deposit(void* h, int fid, uint64_t* host) {
    fields::Grid2D* g = field(static_cast<World*>(h), fid);
    if (!g) return 1;
    std::memcpy(host, g->deposit, sizeof(uint64_t) * static_cast<size_t>(g->n) * g->n);
    return 0;
}

// taumoeba_spawn (src/sim/predation.cu:420-432).
int ref_tau_spawn(void* h, int32_t count, uint64_t seed) {
    World* w = static_cast<World*>(h);
    return static_cast<int>(taumoeba_spawn(w->taumoeba, count, w->chamber, seed).status);
}
int32_t ref_tau_count(void* h) { return static_cast<World*>(h)->taumoeba.count; }
uint64_t ref_tau_next_id(void* h) { return static_cast<World*>(h)->taumoeba.next_id; }
void ref_set_tau_compaction(void* h, int on) { static_cast<World*>(h)->motion.tau_compaction_enabled = on != 0; }

// The predator store's arrays in snapshot order (dir 0: out to host[k], 1: in from host[k]).
int ref_tau_io(void* h, int dir, void** host, int32_t count, uint64_t next_id) {
    TaumoebaStore& t = static_cast<World*>(h)->taumoeba;
    void* d[20] = {t.id, t.flags, t.x, t.y, t.z, t.vx, t.vy, t.vz, t.dir_x, t.dir_y, t.dir_z, t.biomass,
                   t.prey_biomass, t.digest_timer, t.tolerance, t.generation, t.rng_state, t.density_ema,
                   t.run_timer, t.target};
    const size_t sz[20] = {8, 4, 8, 8, 8, 8, 8, 8, 4, 4, 4, 8, 8, 4, 4, 4, 8, 4, 4, 4};
    if (dir == 1) {
        if (count > t.capacity) return 1;
        t.count = count;
        t.next_id = next_id;
    }
    for (int k = 0; k < 20; ++k) {
        const size_t b = sz[k] * static_cast<size_t>(dir == 1 ? count : t.count);
        if (dir == 0) std::memcpy(host[k], d[k], b);
        else std::memcpy(d[k], host[k], b);
    }
    return 0;
}

// World::flash_active / petrova_flash_power and world_flash_audit (src/sim/flash.cu:69-78).
void ref_set_flash(void* h, int active, double power) {
    World* w = static_cast<World*>(h);
    w->flash_active = active != 0;
    if (power > 0.0) w->petrova_flash_power = power;
}
void ref_flash_audit(void* h, double* impulse_ns, double* discharged_j) {
    world_flash_audit(*static_cast<World*>(h), *impulse_ns, *discharged_j);
}

// world_apply_brush (src/sim/step.cu:80-89).
int ref_apply_brush(void* h, int kind, double x, double y, double radius, double strength) {
    return static_cast<int>(world_apply_brush(*static_cast<World*>(h), static_cast<BrushKind>(kind), x, y,
                                              radius, strength).status);
}

void ref_step(void* h, int32_t ticks) {
    World* w = static_cast<World*>(h);
    for (int32_t t = 0; t < ticks; ++t) world_step(*w);
}

// One stage of world_step (src/sim/step.cu:109-184) at the world's dt.
int ref_stage(void* h, int stage) {
    World* w = static_cast<World*>(h);
    const double dt = canon::DT_PHYSICS * w->physics_rate;
    switch (stage) {
        case 0: return static_cast<int>(hash_build(w->hash, w->cells.view, w->cells.count).status);
        case 1: thermal_step(*w, dt); return 0;
        case 2: emission_step(*w, dt); return 0;
        case 3: taxis_step(*w, dt); return 0;
        case 4: motion_step(*w, dt); return 0;
        case 5:
            fields::grid_flush_deposits(w->fields.co2);
            fields::grid_flush_deposits(w->fields.n2);
            fields::grid_diffuse(w->fields.co2, dt);
            fields::grid_diffuse(w->fields.n2, dt);
            return 0;
        case 6: lifecycle_step(*w, dt); return 0;
        case 7: return static_cast<int>(cell_store_compact(w->cells).status);
        case 8: ++w->tick; w->sim_time_s += dt; return 0;
    }
    return 1;
}

// Raw grid operations (src/fields/diffuse.cu:136-186).
int ref_grid_diffuse(void* h, int fid, double dt) {
    return static_cast<int>(fields::grid_diffuse(*field(static_cast<World*>(h), fid), dt).status);
}
int ref_grid_substep(void* h, int fid, double dt_sub) {
    return static_cast<int>(fields::grid_diffuse_substep(*field(static_cast<World*>(h), fid), dt_sub).status);
}
int32_t ref_grid_substeps(void* h, int fid, double dt) {
    const fields::Grid2D* g = field(static_cast<World*>(h), fid);
    return fields::substeps_for_dt(g->dx, g->diffusivity, dt);
}

// Hash buffers after hash_build: dims = {nx, ny, nz, bucket_count}.
void ref_hash_io(void* h, int32_t* dims, uint32_t* keys_sorted, uint32_t* vals_sorted,
                 int32_t* bucket_start, int32_t* bucket_end) {
    const SpatialHash& s = static_cast<World*>(h)->hash;
    dims[0] = s.nx; dims[1] = s.ny; dims[2] = s.nz; dims[3] = s.bucket_count;
    const int32_t n = static_cast<World*>(h)->cells.count;
    if (keys_sorted) std::memcpy(keys_sorted, s.d_keys_sorted, sizeof(uint32_t) * n);
    if (vals_sorted) std::memcpy(vals_sorted, s.d_vals_sorted, sizeof(uint32_t) * n);
    if (bucket_start) std::memcpy(bucket_start, s.d_bucket_start, sizeof(int32_t) * s.bucket_count);
    if (bucket_end) std::memcpy(bucket_end, s.d_bucket_end, sizeof(int32_t) * s.bucket_count);
}

// Forces of the last motion_step (World::d_fx/fy/fz).
void ref_forces(void* h, double* fx, double* fy, double* fz) {
    World* w = static_cast<World*>(h);
    const size_t b = sizeof(double) * static_cast<size_t>(w->cells.count);
    std::memcpy(fx, w->d_fx, b); std::memcpy(fy, w->d_fy, b); std::memcpy(fz, w->d_fz, b);
}

// world_stats (src/sim/stats.cu:102-153) flattened: doubles in Stats order.
void ref_stats(void* h, double* out /* 24 */) {
    const contract::Stats s = world_stats(*static_cast<World*>(h));
    const double v[] = {static_cast<double>(s.tick), s.sim_time_s, double(s.n_live), double(s.n_dead),
                        double(s.n_dormant), double(s.n_awake), double(s.n_taumoeba), s.mean_charge,
                        s.total_energy_j, s.mean_temp_cell_k, s.mean_temp_medium_k,
                        s.max_temp_medium_k, s.co2_total_kg, s.n2_total_kg, s.mean_tau_tolerance,
                        double(s.divisions_this_window), double(s.deaths_this_window),
                        double(s.boil_events), double(s.ignitions_this_window), s.physics_rate,
                        s.biology_rate, double(s.non_canon_run)};
    for (size_t k = 0; k < sizeof(v) / sizeof(v[0]); ++k) out[k] = v[k];
}

// Raw StatsAccum after world_stats: the fixed-point sums, bit for bit.
void ref_stats_accum(void* h, uint64_t* out /* 12 */) {
    const StatsAccum& a = static_cast<World*>(h)->stats_host;
    const uint64_t v[] = {a.energy, a.temp_cell, a.temp_medium, a.co2, a.n2, a.max_temp,
                          a.tau_tolerance, a.n_alive, a.n_dead, a.n_awake, a.n_dormant, a.n_taumoeba};
    for (int k = 0; k < 12; ++k) out[k] = v[k];
}

// Host counters carried by World: {divisions_this_window, deaths_total, dead_slots_prev}.
void ref_counters(void* h, int64_t* out) {
    World* w = static_cast<World*>(h);
    out[0] = w->divisions_this_window; out[1] = w->deaths_total; out[2] = w->dead_slots_prev;
}

// snapshot_to_bytes (src/sim/snapshot.cu:134-165): returns the byte count and
// copies the snapshot into out when cap is large enough; -1 on failure.
int64_t ref_snapshot(void* h, const char* scenario_id, char* out, int64_t cap) {
    std::vector<char> bytes;
    if (snapshot_to_bytes(*static_cast<World*>(h), scenario_id, bytes)) return -1;
    if (out && cap >= (int64_t)bytes.size()) std::memcpy(out, bytes.data(), bytes.size());
    return (int64_t)bytes.size();
}

// snapshot_state_hash (src/sim/snapshot.cu:126-132).
uint64_t ref_state_hash(void* h) {
    uint64_t x = 0;
    if (snapshot_state_hash(*static_cast<World*>(h), x)) return 0;
    return x;
}

// A scenario (the text of a scenarios/*.json file) through the reference's own
// loader and driver (src/sim/scenario.cpp) and accept evaluation
// (src/sim/accept.cpp): instantiate, then `ticks` ticks as the headless
// runner's --assert loop takes them (tools/headless.cpp:197-233: drive, step,
// Stats and aggregates every `stride` ticks, final Stats), then one measured
// value per accept check. Returns the World (for the other ref_* readers; free
// it with ref_world_destroy) or null when the scenario does not parse or build.
void* ref_scenario_run(const char* text, int64_t ticks, double* measured, int32_t* n_checks) {
    static contract::Scenario sc;
    if (scenario_parse(std::string(text), sc)) return nullptr;
    World* w = new (std::nothrow) World{};
    if (!w) return nullptr;
    if (scenario_instantiate(sc, *w)) { delete w; return nullptr; }
    const int64_t stride = ticks > 2000 ? ticks / 2000 : 1;
    const MetricNeeds needs = metric_needs(sc);
    RunAggregates agg;
    contract::Stats st{};
    for (int64_t t = 0; t < ticks; ++t) {
        scenario_apply_drive(*w, sc);
        world_step(*w);
        if (t % stride == 0) {
            st = world_stats(*w);
            aggregates_sample(agg, st, *w, needs, 2.0, 4.0);
        }
    }
    st = world_stats(*w);
    aggregates_sample(agg, st, *w, needs, 2.0, 4.0);
    for (int i = 0; i < sc.accept_count; ++i) measured[i] = metric_measure(sc.accept[i].metric, st, agg, *w, sc);
    *n_checks = sc.accept_count;
    return w;
}

}  // extern "C"
