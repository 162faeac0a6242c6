// astro_sim_gb -- the reference simulator's World API implemented over the
// engine's C ABI (include/agb.h), so that code written against the reference's
// src/sim (its tools and tests) links against the engine instead of src/sim +
// src/fields. It is compiled against the reference's own headers, which declare
// the types and the functions defined here:
//
//   world_create / world_destroy / world_step / world_sim_time /
//   clock_preset_rates / world_set_clock / world_stats / world_apply_brush /
//   world_flash_audit           (src/sim/world.cuh:183-243)
//   cell_store_spawn / cell_store_set_charge / cell_store_download_positions /
//   cell_store_download_velocities / cell_store_download_energy
//                               (src/sim/cell_store.cuh:73-106)
//   grid_fill / grid_download / grid_brush, for a world's own fields
//                               (src/fields/grid.cuh:91-103)
//   taumoeba_spawn / taumoeba_download_*   (src/sim/predation.cuh:133-141)
//   snapshot_to_bytes / snapshot_from_bytes / snapshot_save / snapshot_load /
//   snapshot_state_hash         (src/sim/snapshot.h:20-37)
//
// The engine's world lives behind the reference's World object, and the World's
// public members that callers read or set between ticks are kept in step:
//   * before a tick, the clock (physics_rate, biology_rate, unclamped as the
//     reference's tick reads them), the directional light and ambient
//     irradiance, the flash arming, the live overrides (co2_mass_per_division,
//     petrova_max_power) and each field's boundary kind (Grid2D::bc) go to the
//     engine when they changed since the last tick;
//   * after create, spawn and every tick (one synchronisation), the cell
//     store's view (its 25 device SoA pointers, count and capacity), count and
//     next id, and the death and division counters come from it, and the tick
//     and the simulated time
//     advance as the reference advances them. The view points into the
//     engine's device arrays (callers may read and write them between ticks)
//     and stays valid until the next tick (compaction swaps them);
//   * the four Grid2D fields carry the reference's metadata (n, extent, dx,
//     diffusivity, ambient, deposit scale, Robin coefficient, substeps, bc);
//     their device pointers stay null, because the engine ping-pongs its field
//     buffers inside the tick: read and write them with grid_download/grid_fill.
//   * the predator store mirrors its count, capacity and next id; its device
//     pointers stay null (read predators with taumoeba_download_*).
// Not provided: the stage functions (motion_step, thermal_step, ...) and the
// lower-level stores (hash_*, grid_create/diffuse, cell_store_create/destroy/
// compact/sample, taumoeba_create/destroy/compact): the engine runs the whole
// tick as one captured graph and owns its stores. The reference's own
// scenario loader and acceptance code (src/sim/scenario.cpp, accept.cpp) and
// tools/headless.cpp compile against these unchanged.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "agb.h"
#include "contracts/snapshot_v1.h"
#include "core/canon_generated.h"
#include "sim/cell_store.cuh"
#include "sim/predation.cuh"
#include "sim/snapshot.h"
#include "sim/world.cuh"

namespace {

struct Binding {
    agb_world* h = nullptr;
    int32_t tau_capacity = 0;
    double physics = 1.0, biology = 1.0;   // last rates pushed
    agb_light light{};                     // last light pushed
    bool flash = false;
    double flash_power = 0.0;
    double quota = 0.0, max_power = 0.0;   // last overrides pushed
    int32_t bc[AGB_FIELD_COUNT] = {};      // last boundary kind pushed per field
    double face[AGB_FIELD_COUNT] = {};     // its face value (the field's ambient)
};

struct GridKey {
    Binding* b;
    int32_t field;
};

std::mutex g_mu;
std::map<const void*, Binding*> g_by_world;    // World* -> binding
std::map<const void*, Binding*> g_by_cells;    // &World::cells -> binding
std::map<const void*, GridKey> g_by_grid;      // &World::fields.<field> -> binding, field
std::map<const void*, Binding*> g_by_tau;       // &World::taumoeba -> binding

astro::fields::Grid2D* world_grid(astro::sim::World& w, int32_t f) {
    switch (f) {
        case AGB_FIELD_TEMPERATURE: return &w.fields.temperature;
        case AGB_FIELD_CO2: return &w.fields.co2;
        case AGB_FIELD_N2: return &w.fields.n2;
        default: return &w.fields.irradiance;
    }
}

bool grid_of(const void* g, GridKey& out) {
    std::lock_guard<std::mutex> lock(g_mu);
    const auto it = g_by_grid.find(g);
    if (it == g_by_grid.end()) return false;
    out = it->second;
    return true;
}

// grid_create's metadata (diffuse.cu:91-105) for a field the engine holds.
void grid_meta(astro::fields::Grid2D& g, const agb_grid_desc& gd, double extent) {
    g = astro::fields::Grid2D{};
    if (gd.nx <= 0) return;
    g.n = gd.nx;
    g.extent = extent;
    g.dx = extent / (double)gd.nx;
    g.diffusivity = gd.diffusivity;
    g.ambient = gd.init;
    g.deposit_scale = gd.deposit_scale;
    g.robin_coeff = g.dx * astro::canon::AIR_CONVECTION_H / astro::canon::WATER_CONDUCTIVITY;
    g.substeps = (int32_t)(astro::canon::DT_PHYSICS / (g.dx * g.dx / (4.0 * gd.diffusivity))) + 1;
    g.bc = static_cast<astro::contract::BoundaryCondition>(gd.bc[0]);
}

Binding* binding_of(const void* key, const std::map<const void*, Binding*>& m) {
    std::lock_guard<std::mutex> lock(g_mu);
    const auto it = m.find(key);
    return it == m.end() ? nullptr : it->second;
}

astro::Error status_error(agb_status rc, const char* what) {
    if (rc == AGB_OK) return astro::ok();
    // agb_status 0-9 are astro::Status 0-9; a bounded device wait that expired
    // reports as a CUDA error.
    const int32_t s = rc <= AGB_UNSUPPORTED ? (int32_t)rc : (int32_t)astro::Status::CudaError;
    return astro::fail(static_cast<astro::Status>(s), what);
}

// The cell store's public members from the engine.
void pull_cells(astro::sim::World& w, agb_world* h) {
    agb_cells v{};
    if (agb_world_device_cells(h, &v) != AGB_OK) return;
    static_assert(sizeof(agb_cells) == sizeof(astro::contract::CellStoreView), "agb_cells is CellStoreView");
    std::memcpy(&w.cells.view, &v, sizeof(v));
    w.cells.count = v.count;
    w.cells.capacity = v.capacity;
    agb_cells none{};                                  // no arrays: count and next id only
    int32_t cnt = 0;
    uint64_t nid = 0;
    if (agb_world_export_cells(h, &none, 0, &cnt, &nid, nullptr) == AGB_OK) w.cells.next_id = nid;
}

// The predator store's count, capacity and next id (predation.cuh:85-106).
void pull_tau(astro::sim::World& w, agb_world* h, int32_t capacity) {
    agb_taumoeba none{};
    int32_t n = 0;
    uint64_t nid = 1;
    if (agb_world_export_taumoeba(h, &none, 0, &n, &nid, nullptr) != AGB_OK) return;
    w.taumoeba.count = n;
    w.taumoeba.capacity = capacity;
    w.taumoeba.next_id = nid;
}

// Everything world_step refreshes, with one synchronisation (agb_world_mirror).
void pull_all(astro::sim::World& w, Binding* b) {
    agb_mirror m{};
    if (agb_world_mirror(b->h, &m, nullptr) != AGB_OK) return;
    std::memcpy(&w.cells.view, &m.cells, sizeof(m.cells));
    w.cells.count = m.cells.count;
    w.cells.capacity = m.cells.capacity;
    w.cells.next_id = m.next_id;
    w.divisions_this_window = (int32_t)m.divisions_this_window;
    w.deaths_total = m.deaths_total;
    w.dead_slots_prev = (int32_t)m.dead_slots_prev;
    w.taumoeba.count = m.tau_count;
    w.taumoeba.capacity = b->tau_capacity;
    w.taumoeba.next_id = m.tau_next_id;
}

// The World's knobs that callers set by assignment, pushed when they changed.
void push_knobs(astro::sim::World& w, Binding* b) {
    if (w.physics_rate != b->physics || w.biology_rate != b->biology) {
        agb_world_set_rates(b->h, w.physics_rate, w.biology_rate);
        b->physics = w.physics_rate;
        b->biology = w.biology_rate;
    }
    agb_light L{};
    L.dir_x = w.light.dir_x;
    L.dir_y = w.light.dir_y;
    L.dir_z = 0.0f;
    L.irradiance = w.light.irradiance;
    L.ambient = w.ambient_irradiance;
    L.enabled = w.light.enabled;
    if (std::memcmp(&L, &b->light, sizeof(L)) != 0) {
        agb_world_set_light(b->h, &L);
        b->light = L;
    }
    if (w.flash_active != b->flash || w.petrova_flash_power != b->flash_power) {
        agb_world_set_flash(b->h, w.flash_active ? 1 : 0, w.petrova_flash_power);
        b->flash = w.flash_active;
        b->flash_power = w.petrova_flash_power;
    }
    if (w.co2_mass_per_division != b->quota || w.petrova_max_power != b->max_power) {
        agb_world_set_overrides(b->h, w.co2_mass_per_division, w.petrova_max_power);
        b->quota = w.co2_mass_per_division;
        b->max_power = w.petrova_max_power;
    }
    // A Grid2D has one boundary kind for its four sides; the engine's depth-
    // averaged grid has no z faces to speak of, so all six follow it.
    for (int32_t f = 0; f < AGB_FIELD_COUNT; ++f) {
        const astro::fields::Grid2D& g = *world_grid(w, f);
        if (g.n <= 0 || (int32_t)g.bc == b->bc[f]) continue;
        int32_t bc[6];
        double face[6];
        for (int k = 0; k < 6; ++k) { bc[k] = (int32_t)g.bc; face[k] = b->face[f]; }
        if (agb_world_set_boundary(b->h, f, bc, face) == AGB_OK) b->bc[f] = (int32_t)g.bc;
    }
}

}  // namespace

namespace astro::sim {

namespace {

// world_create's descriptor (step.cu:9-78) in the engine's terms.
agb_world_desc engine_desc(const WorldDesc& d) {
    agb_world_desc a;
    agb_world_desc_default(&a);
    a.chamber_w = d.chamber.w;
    a.chamber_h = d.chamber.h;
    a.chamber_d = d.chamber.d;
    a.capacity = d.capacity > 0 ? d.capacity : canon::DEFAULT_CELLS;    // step.cu:10
    a.tau_capacity = d.tau_capacity;
    a.seed = d.seed;
    const MotionConfig& m = d.motion;
    a.boundary_x = (int32_t)m.boundary_x;
    a.boundary_y = (int32_t)m.boundary_y;
    a.gravity_axis = (int32_t)m.gravity_axis;
    a.thermal_noise = m.thermal_noise;
    a.contact_enabled = m.contact_enabled;
    a.adhesion_enabled = m.adhesion_enabled;
    a.thermal_enabled = m.thermal_enabled;
    a.emission_enabled = m.emission_enabled;
    a.taxis_enabled = m.taxis_enabled;
    a.occlusion_exact = m.occlusion_exact;
    a.ambient_temp = m.ambient_temp;
    a.store_disposition = (int32_t)m.store_disposition;
    a.compaction_enabled = m.compaction_enabled;
    a.tau_compaction_enabled = m.tau_compaction_enabled;
    // The temperature grid starts at the ambient temperature, CO2 at co2_init
    // (step.cu:29-36), their faces at the same values.
    a.grid[AGB_FIELD_TEMPERATURE].init = m.ambient_temp;
    a.grid[AGB_FIELD_CO2].init = d.co2_init;
    for (int k = 0; k < 6; ++k) {
        a.grid[AGB_FIELD_TEMPERATURE].face_value[k] = m.ambient_temp;
        a.grid[AGB_FIELD_CO2].face_value[k] = d.co2_init;
    }
    return a;
}

// Ties the engine world h to w and mirrors its state into w's members.
void bind(World& w, const WorldDesc& d, const agb_world_desc& a, agb_world* h) {
    Binding* b = new Binding();
    b->tau_capacity = a.tau_capacity > 0 ? a.tau_capacity : canon::DEFAULT_TAUMOEBA;
    b->light = a.light;                                // what the engine starts with
    b->flash_power = canon::PETROVA_FLASH_POWER;
    b->h = h;
    b->quota = a.co2_mass_per_division;
    b->max_power = a.max_emit_power;
    for (int32_t f = 0; f < AGB_FIELD_COUNT; ++f) {
        grid_meta(*world_grid(w, f), a.grid[f], d.chamber.w);
        b->bc[f] = a.grid[f].bc[0];
        b->face[f] = a.grid[f].face_value[0];
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_by_world[&w] = b;
        g_by_cells[&w.cells] = b;
        g_by_tau[&w.taumoeba] = b;
        for (int32_t f = 0; f < AGB_FIELD_COUNT; ++f) g_by_grid[world_grid(w, f)] = GridKey{b, f};
    }
    w.chamber = d.chamber;
    w.motion = d.motion;
    w.seed = d.seed;
    w.tick = 0;
    w.sim_time_s = 0.0;
    w.physics_rate = 1.0;
    w.biology_rate = 1.0;
    w.cells.next_id = 1;
    pull_cells(w, h);
    pull_tau(w, h, b->tau_capacity);
}

}  // namespace

Error world_create(World& w, const WorldDesc& d) {
    const agb_world_desc a = engine_desc(d);
    agb_world* h = nullptr;
    const agb_status rc = agb_world_create(&a, &h);
    if (rc != AGB_OK) return status_error(rc, "agb_world_create");
    bind(w, d, a, h);
    return ok();
}

void world_destroy(World& w) {
    Binding* b = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        const auto it = g_by_world.find(&w);
        if (it != g_by_world.end()) {
            b = it->second;
            g_by_world.erase(it);
            g_by_cells.erase(&w.cells);
            g_by_tau.erase(&w.taumoeba);
            for (int32_t f = 0; f < AGB_FIELD_COUNT; ++f) g_by_grid.erase(world_grid(w, f));
        }
    }
    if (b) {
        agb_world_destroy(b->h);
        delete b;
    }
    w = World{};
}

void world_step(World& w) {
    Binding* b = binding_of(&w, g_by_world);
    if (!b) return;
    push_knobs(w, b);
    agb_world_step_graph(b->h, 1, nullptr);
    pull_all(w, b);
    ++w.tick;                                          // the clock as step.cu advances it
    w.sim_time_s += canon::DT_PHYSICS * w.physics_rate;
}

double world_sim_time(const World& w) { return w.sim_time_s; }

void clock_preset_rates(contract::ClockPreset preset, double& physics, double& biology) {
    switch (preset) {                                  // step.cu:190-203
        case contract::ClockPreset::Motion:
            physics = canon::CLOCK_MOTION_PHYSICS; biology = canon::CLOCK_MOTION_BIOLOGY; break;
        case contract::ClockPreset::Metabolic:
            physics = canon::CLOCK_METABOLIC_PHYSICS; biology = canon::CLOCK_METABOLIC_BIOLOGY; break;
        case contract::ClockPreset::Generational:
            physics = canon::CLOCK_GENERATIONAL_PHYSICS; biology = canon::CLOCK_GENERATIONAL_BIOLOGY; break;
        default:
            physics = canon::CLOCK_REALTIME_PHYSICS; biology = canon::CLOCK_REALTIME_BIOLOGY; break;
    }
}

void world_set_clock(World& w, contract::ClockPreset preset, double custom_physics, double custom_biology) {
    double p = custom_physics, q = custom_biology;
    if (preset != contract::ClockPreset::Custom) clock_preset_rates(preset, p, q);
    w.physics_rate = p < canon::CLOCK_PHYSICS_MIN ? canon::CLOCK_PHYSICS_MIN
                   : (p > canon::CLOCK_PHYSICS_MAX ? canon::CLOCK_PHYSICS_MAX : p);
    w.biology_rate = q < canon::CLOCK_BIOLOGY_MIN ? canon::CLOCK_BIOLOGY_MIN
                   : (q > canon::CLOCK_BIOLOGY_MAX ? canon::CLOCK_BIOLOGY_MAX : q);
    if (Binding* b = binding_of(&w, g_by_world)) push_knobs(w, b);
}

contract::Stats world_stats(World& w) {
    contract::Stats out{};
    Binding* b = binding_of(&w, g_by_world);
    if (!b) return out;
    agb_stats st{};
    static_assert(sizeof(agb_stats) == sizeof(contract::Stats), "agb_stats is Stats");
    if (agb_world_stats(b->h, &st, nullptr) == AGB_OK) std::memcpy(&out, &st, sizeof(out));
    w.divisions_this_window = 0;
    return out;
}

Error world_apply_brush(World& w, BrushKind kind, double x, double y, double radius, double strength) {
    Binding* b = binding_of(&w, g_by_world);
    if (!b) return fail(Status::InvalidArgument, "world not created by the engine");
    return status_error(agb_world_apply_brush(b->h, (int32_t)kind, x, y, radius, strength, nullptr),
                        "agb_world_apply_brush");
}

void world_flash_audit(const World& w, double& impulse_ns, double& discharged_j) {
    impulse_ns = discharged_j = 0.0;
    if (Binding* b = binding_of(&w, g_by_world)) agb_world_flash_audit(b->h, &impulse_ns, &discharged_j);
}

Error cell_store_spawn(CellStore& s, const SpawnParams& p, const Chamber& c, uint64_t seed) {
    (void)c;                                           // the engine's world carries the chamber
    Binding* b = binding_of(&s, g_by_cells);
    if (!b) return fail(Status::InvalidArgument, "cell store not created by the engine");
    agb_spawn a{};
    a.count = p.count;
    a.placement = (int32_t)p.placement;
    a.charge_dist = (int32_t)p.charge_dist;
    a.awake = p.awake ? 1 : 0;
    a.place_x = p.place_x;
    a.place_y = p.place_y;
    a.place_radius = p.place_radius;
    a.charge_a = p.charge_a;
    a.charge_b = p.charge_b;
    const agb_status rc = agb_world_spawn_seeded(b->h, &a, seed, nullptr);
    if (rc != AGB_OK) return status_error(rc, "agb_world_spawn_seeded");
    agb_cells v{};
    int32_t cnt = 0;
    uint64_t nid = 0;
    agb_world_export_cells(b->h, &v, 0, &cnt, &nid, nullptr);    // count and next id only
    s.next_id = nid;
    agb_cells dv{};
    if (agb_world_device_cells(b->h, &dv) == AGB_OK) {
        std::memcpy(&s.view, &dv, sizeof(dv));
        s.count = dv.count;
        s.capacity = dv.capacity;
    }
    return ok();
}

Error cell_store_set_charge(CellStore& s, double charge) {
    Binding* b = binding_of(&s, g_by_cells);
    if (!b) return fail(Status::InvalidArgument, "cell store not created by the engine");
    if (s.count <= 0) return ok();
    return status_error(agb_world_set_charge(b->h, charge, nullptr), "agb_world_set_charge");
}

namespace {

// Full device-to-host copies of three double columns (cell_store.cu:301-330).
Error copy_columns(const double* const* src, double* const* dst, int ncol, int32_t count, int32_t max_count,
                   const char* what) {
    const int32_t n = count < max_count ? count : max_count;
    if (n <= 0) return ok();
    for (int k = 0; k < ncol; ++k) {
        const cudaError_t e = cudaMemcpy(dst[k], src[k], sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(Status::CudaError, what);
    }
    return ok();
}

}  // namespace

Error cell_store_download_positions(const CellStore& s, double* x, double* y, double* z, int32_t max_count) {
    const double* src[3] = {s.view.x, s.view.y, s.view.z};
    double* dst[3] = {x, y, z};
    return copy_columns(src, dst, 3, s.count, max_count, "download positions");
}

Error cell_store_download_velocities(const CellStore& s, double* vx, double* vy, double* vz, int32_t max_count) {
    const double* src[3] = {s.view.vx, s.view.vy, s.view.vz};
    double* dst[3] = {vx, vy, vz};
    return copy_columns(src, dst, 3, s.count, max_count, "download velocities");
}

Error cell_store_download_energy(const CellStore& s, double* energy, int32_t max_count) {
    const double* src[1] = {s.view.energy};
    double* dst[1] = {energy};
    return copy_columns(src, dst, 1, s.count, max_count, "download energy");
}

namespace {

// One predator array, copied out through the engine (taumoeba_download_*).
template <class T>
Error tau_column(const TaumoebaStore& s, T* out, int32_t max_count, T* agb_taumoeba::* col, const char* what) {
    Binding* b = binding_of(&s, g_by_tau);
    if (!b) return fail(Status::InvalidArgument, "predator store not created by the engine");
    const int32_t n = s.count < max_count ? s.count : max_count;
    if (n <= 0) return ok();
    agb_taumoeba dst{};
    dst.*col = out;
    int32_t cnt = 0;
    uint64_t nid = 0;
    return status_error(agb_world_export_taumoeba(b->h, &dst, n, &cnt, &nid, nullptr), what);
}

}  // namespace

Error taumoeba_spawn(TaumoebaStore& s, int32_t count, const Chamber& c, uint64_t seed) {
    (void)c;                                           // the engine's world carries the chamber
    Binding* b = binding_of(&s, g_by_tau);
    if (!b) return fail(Status::InvalidArgument, "predator store not created by the engine");
    if (count <= 0) return ok();
    const agb_status rc = agb_world_spawn_taumoeba(b->h, count, seed, nullptr);
    if (rc != AGB_OK) return status_error(rc, "agb_world_spawn_taumoeba");
    agb_taumoeba none{};
    int32_t n = 0;
    uint64_t nid = 1;
    if (agb_world_export_taumoeba(b->h, &none, 0, &n, &nid, nullptr) == AGB_OK) {
        s.count = n;
        s.next_id = nid;
    }
    return ok();
}

Error taumoeba_download_positions(const TaumoebaStore& s, double* x, double* y, double* z, int32_t max_count) {
    if (Error e = tau_column(s, x, max_count, &agb_taumoeba::x, "taumoeba positions")) return e;
    if (Error e = tau_column(s, y, max_count, &agb_taumoeba::y, "taumoeba positions")) return e;
    return tau_column(s, z, max_count, &agb_taumoeba::z, "taumoeba positions");
}
Error taumoeba_download_biomass(const TaumoebaStore& s, double* biomass, int32_t max_count) {
    return tau_column(s, biomass, max_count, &agb_taumoeba::biomass, "taumoeba biomass");
}
Error taumoeba_download_tolerance(const TaumoebaStore& s, float* tolerance, int32_t max_count) {
    return tau_column(s, tolerance, max_count, &agb_taumoeba::tolerance, "taumoeba tolerance");
}
Error taumoeba_download_generation(const TaumoebaStore& s, uint32_t* generation, int32_t max_count) {
    return tau_column(s, generation, max_count, &agb_taumoeba::generation, "taumoeba generation");
}
Error taumoeba_download_flags(const TaumoebaStore& s, uint32_t* flags, int32_t max_count) {
    return tau_column(s, flags, max_count, &agb_taumoeba::flags, "taumoeba flags");
}

// Snapshots (snapshot.cu:134-262): the engine writes and reads the same file
// layout; the World's knobs go to the engine first so the bytes carry them.
Error snapshot_to_bytes(const World& w, const char* scenario_id, std::vector<char>& out) {
    Binding* b = binding_of(&w, g_by_world);
    if (!b) return fail(Status::InvalidArgument, "world not created by the engine");
    push_knobs(const_cast<World&>(w), b);
    int64_t size = 0;
    agb_status rc = agb_world_snapshot_save(b->h, scenario_id, nullptr, 0, &size, nullptr);
    if (rc != AGB_OK) return status_error(rc, "agb_world_snapshot_save");
    out.resize((size_t)size);
    rc = agb_world_snapshot_save(b->h, scenario_id, out.data(), size, &size, nullptr);
    return status_error(rc, "agb_world_snapshot_save");
}

Error snapshot_from_bytes(const char* data, size_t n, World& w) {
    if (n < sizeof(contract::SnapshotHeader)) return fail(Status::FileIoError, "snapshot: too small");
    contract::SnapshotHeader hd{};
    std::memcpy(&hd, data, sizeof(hd));
    // The world is created from the header's chamber, capacities and seed with
    // the default motion configuration, as the reference does.
    WorldDesc d;
    d.chamber = Chamber{hd.chamber_w, hd.chamber_h, hd.chamber_d};
    d.capacity = hd.cell_capacity;
    d.tau_capacity = hd.taumoeba_capacity;
    d.seed = hd.seed;
    if (binding_of(&w, g_by_world)) world_destroy(w);
    const agb_world_desc a = engine_desc(d);
    agb_world* h = nullptr;
    const agb_status rc = agb_world_snapshot_load(&a, data, (int64_t)n, &h);
    if (rc != AGB_OK) return status_error(rc, "agb_world_snapshot_load");
    bind(w, d, a, h);
    Binding* b = binding_of(&w, g_by_world);
    // Overrides come first in the body (OVERRIDE_FIELDS, snapshot.cu:79-83).
    const char* cur = data + sizeof(hd);
    for (int32_t i = 0; i < hd.override_count && cur + sizeof(contract::ParamOverride) <= data + n; ++i) {
        contract::ParamOverride ov{};
        std::memcpy(&ov, cur, sizeof(ov));
        cur += sizeof(ov);
        if (std::strncmp(ov.key, "PETROVA_MAX_POWER", sizeof(ov.key)) == 0) w.petrova_max_power = b->max_power = ov.value;
        if (std::strncmp(ov.key, "PETROVA_FLASH_POWER", sizeof(ov.key)) == 0) w.petrova_flash_power = b->flash_power = ov.value;
        if (std::strncmp(ov.key, "CO2_MASS_PER_DIVISION", sizeof(ov.key)) == 0) w.co2_mass_per_division = b->quota = ov.value;
    }
    w.seed = hd.seed;
    w.tick = hd.tick;
    w.sim_time_s = hd.sim_time_s;
    w.physics_rate = b->physics = hd.physics_rate;
    w.biology_rate = b->biology = hd.biology_rate;
    w.non_canon_run = hd.non_canon_run != 0;
    w.cells.next_id = hd.next_cell_id;
    return ok();
}

Error snapshot_save(const World& w, const char* path, const char* scenario_id) {
    std::vector<char> bytes;
    if (Error e = snapshot_to_bytes(w, scenario_id, bytes)) return e;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(Status::FileIoError, "snapshot: cannot open file for write");
    const bool wrote = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    std::fclose(f);
    return wrote ? ok() : fail(Status::FileIoError, "snapshot: write failed");
}

Error snapshot_load(const char* path, World& w) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(Status::FileIoError, "snapshot: cannot open file for read");
    std::vector<char> all;
    char buf[65536];
    size_t r = 0;
    while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) all.insert(all.end(), buf, buf + r);
    std::fclose(f);
    return snapshot_from_bytes(all.data(), all.size(), w);
}

Error snapshot_state_hash(const World& w, uint64_t& hash_out) {
    Binding* b = binding_of(&w, g_by_world);
    if (!b) return fail(Status::InvalidArgument, "world not created by the engine");
    push_knobs(const_cast<World&>(w), b);
    return status_error(agb_world_state_hash(b->h, &hash_out, nullptr), "agb_world_state_hash");
}

}  // namespace astro::sim

namespace astro::fields {

Error grid_fill(Grid2D& g, float value) {
    GridKey k;
    if (!grid_of(&g, k)) return fail(Status::InvalidArgument, "grid not held by an engine world");
    std::vector<float> v((size_t)g.n * (size_t)g.n, value);
    const agb_status rc = agb_world_import_field(k.b->h, k.field, v.data(), nullptr);
    return rc == AGB_OK ? ok() : fail(Status::CudaError, "agb_world_import_field");
}

Error grid_download(const Grid2D& g, float* out) {
    GridKey k;
    if (!grid_of(&g, k)) return fail(Status::InvalidArgument, "grid not held by an engine world");
    const agb_status rc = agb_world_export_field(k.b->h, k.field, out, nullptr);
    return rc == AGB_OK ? ok() : fail(Status::CudaError, "agb_world_export_field");
}

// grid_brush on one of a world's fields: the engine's brush adds `amount` over
// the disc (the kind only picks the field, so heat adds and the sign is the
// caller's).
Error grid_brush(Grid2D& g, double x, double y, double radius, double amount) {
    GridKey k;
    if (!grid_of(&g, k)) return fail(Status::InvalidArgument, "grid not held by an engine world");
    int32_t kind;
    switch (k.field) {
        case AGB_FIELD_TEMPERATURE: kind = AGB_BRUSH_HEAT; break;
        case AGB_FIELD_CO2: kind = AGB_BRUSH_INJECT_CO2; break;
        case AGB_FIELD_N2: kind = AGB_BRUSH_INJECT_N2; break;
        default: return fail(Status::InvalidArgument, "no brush on the irradiance field");
    }
    return status_error(agb_world_apply_brush(k.b->h, kind, x, y, radius, amount, nullptr), "agb_world_apply_brush");
}

}  // namespace astro::fields
