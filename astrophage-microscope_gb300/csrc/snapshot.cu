// snapshot.cu -- full-state snapshots in the reference's file format and its
// FNV-1a state hash (contracts/snapshot_v1.h:17-63, src/sim/snapshot.cu:100-246).
//
// Layout: a 256-byte header, then the body the hash covers: parameter
// overrides, the 25 cell arrays in contract order (count elements each), the
// predator arrays (none here: this engine has no predator store, so the
// count is 0 and they add nothing), then the temperature, CO2 and N2 values
// (irradiance is rebuilt every tick and never stored). An nz == 1 world
// writes the reference's bytes exactly; a 3-D grid writes all nx*ny*nz
// values with the header's n_* holding nx.
//
// The body is assembled by one device-to-host copy per array straight into
// the caller's buffer; FNV-1a is a byte-serial recurrence, so it runs on the
// host over the assembled body.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "world_impl.cuh"

namespace {

static_assert(sizeof(agb_snapshot_header) == 256, "snapshot header is 256 bytes (contracts/snapshot_v1.h)");
static_assert(sizeof(agb_param_override) == 56, "override record is 56 bytes");

constexpr size_t kElem[25] = {8, 4, 1, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 8, 8, 4, 8, 4, 4, 4, 4, 4, 4};

// The overrides this engine carries, in the reference's order
// (OVERRIDE_FIELDS, src/sim/snapshot.cu:79-83): the emission cap, the flash
// power and the division quota, each when it differs from canon.
std::vector<agb_param_override> overrides(const agb_world* w) {
    std::vector<agb_param_override> out;
    auto add = [&](const char* key, double value) {
        agb_param_override ov;
        std::memset(&ov, 0, sizeof(ov));           // the key's padding is hashed
        std::strncpy(ov.key, key, sizeof(ov.key) - 1);
        ov.value = value;
        out.push_back(ov);
    };
    const double pmax = w->d.max_emit_power > 0.0 ? w->d.max_emit_power : AGB_PETROVA_MAX_POWER;
    if (pmax != AGB_PETROVA_MAX_POWER) add("PETROVA_MAX_POWER", pmax);
    if (w->flash_power != AGB_PETROVA_FLASH_POWER) add("PETROVA_FLASH_POWER", w->flash_power);
    if (w->d.co2_mass_per_division != AGB_CO2_MASS_PER_DIVISION) add("CO2_MASS_PER_DIVISION", w->d.co2_mass_per_division);
    return out;
}

const int kStoredFields[3] = {AGB_FIELD_TEMPERATURE, AGB_FIELD_CO2, AGB_FIELD_N2};

// The predator store's 20 arrays (collect_tau_spans, snapshot.cu:59-67).
const size_t kTauElem[20] = {8, 4, 8, 8, 8, 8, 8, 8, 4, 4, 4, 8, 8, 4, 4, 4, 8, 4, 4, 4};

void tau_arrays(const TauSoA& t, void* p[20]) {
    void* q[20] = {t.id, t.flags, t.x, t.y, t.z, t.vx, t.vy, t.vz, t.dir_x, t.dir_y, t.dir_z, t.biomass,
                   t.prey_biomass, t.digest_timer, t.tolerance, t.generation, t.rng_state, t.density_ema,
                   t.run_timer, t.target};
    std::memcpy(p, q, sizeof(q));
}

agb_status read_tau_state(agb_world* w, TauState& ts, cudaStream_t s) {
    if (cudaMemcpyAsync(&ts, w->tS, sizeof(TauState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return AGB_CUDA_ERROR;
    return AGB_OK;
}

int64_t body_bytes(const agb_world* w, int32_t count, int32_t tau_count, size_t n_overrides) {
    int64_t b = (int64_t)(n_overrides * sizeof(agb_param_override));
    for (size_t e : kElem) b += (int64_t)e * count;
    for (size_t e : kTauElem) b += (int64_t)e * tau_count;
    for (int f : kStoredFields)
        if (w->c.g[f].enabled) b += 4 * w->c.g[f].count;
    return b;
}

void cell_arrays(const SoA& v, void* p[25]) {
    void* q[25] = {v.id, v.flags, v.death_cause, v.x, v.y, v.z, v.vx, v.vy, v.vz, v.energy,
                   v.temp_cell, v.emit_power, v.dir_x, v.dir_y, v.dir_z, v.biomass, v.co2_held,
                   v.age_s, v.rng_state, v.taxis_memory, v.run_timer, v.t_local, v.irradiance,
                   v.co2_local, v.n2_local};
    std::memcpy(p, q, sizeof(q));
}

agb_status read_dev_state(agb_world* w, DevState& st, cudaStream_t s) {
    if (cudaMemcpyAsync(&st, w->S, sizeof(DevState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return AGB_CUDA_ERROR;
    return AGB_OK;
}

// Body into dst (which holds body_bytes); returns the overrides written.
agb_status write_body(agb_world* w, const DevState& st, const TauState& ts, char* dst, cudaStream_t s,
                      int32_t* n_over) {
    const std::vector<agb_param_override> ov = overrides(w);
    char* p = dst;
    if (!ov.empty()) {
        std::memcpy(p, ov.data(), ov.size() * sizeof(agb_param_override));
        p += ov.size() * sizeof(agb_param_override);
    }
    void* arr[25];
    cell_arrays(st.cur, arr);
    const size_t n = (size_t)st.count;
    for (int k = 0; k < 25; ++k) {
        if (n && cudaMemcpyAsync(p, arr[k], kElem[k] * n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return AGB_CUDA_ERROR;
        p += kElem[k] * n;
    }
    void* tarr[20];
    tau_arrays(ts.cur, tarr);
    const size_t nt = (size_t)ts.count;
    for (int k = 0; k < 20; ++k) {
        if (nt && cudaMemcpyAsync(p, tarr[k], kTauElem[k] * nt, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return AGB_CUDA_ERROR;
        p += kTauElem[k] * nt;
    }
    for (int f : kStoredFields) {
        const GridDev& g = w->c.g[f];
        if (!g.enabled) continue;
        if (cudaMemcpyAsync(p, w->gbuf[f][w->gcur[f]], 4 * (size_t)g.count, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
            return AGB_CUDA_ERROR;
        p += 4 * (size_t)g.count;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return AGB_CUDA_ERROR;
    *n_over = (int32_t)ov.size();
    return AGB_OK;
}

}  // namespace

extern "C" {

uint64_t agb_fnv1a64(const void* data, uint64_t n, uint64_t h) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (uint64_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

agb_status agb_world_state_hash(agb_world* w, uint64_t* hash, agb_stream stream) {
    if (!w || !hash) return AGB_INVALID_ARGUMENT;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    DevState st;
    TauState ts;
    if (read_dev_state(w, st, s) != AGB_OK || read_tau_state(w, ts, s) != AGB_OK) return AGB_CUDA_ERROR;
    std::vector<char> body((size_t)body_bytes(w, st.count, ts.count, overrides(w).size()));
    int32_t n_over = 0;
    const agb_status rc = write_body(w, st, ts, body.data(), s, &n_over);
    if (rc != AGB_OK) return rc;
    *hash = agb_fnv1a64(body.data(), body.size(), AGB_FNV1A64_OFFSET);
    return AGB_OK;
}

agb_status agb_world_snapshot_save(agb_world* w, const char* scenario_id, void* buf, int64_t cap,
                                   int64_t* size, agb_stream stream) {
    if (!w || !size) return AGB_INVALID_ARGUMENT;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    DevState st;
    TauState ts;
    if (read_dev_state(w, st, s) != AGB_OK || read_tau_state(w, ts, s) != AGB_OK) return AGB_CUDA_ERROR;
    const int64_t body = body_bytes(w, st.count, ts.count, overrides(w).size());
    *size = (int64_t)sizeof(agb_snapshot_header) + body;
    if (!buf) return AGB_OK;                            // size query
    if (cap < *size) return AGB_CAPACITY_EXCEEDED;
    char* out = static_cast<char*>(buf);
    int32_t n_over = 0;
    const agb_status rc = write_body(w, st, ts, out + sizeof(agb_snapshot_header), s, &n_over);
    if (rc != AGB_OK) return rc;
    agb_snapshot_header h;
    std::memset(&h, 0, sizeof(h));
    h.magic = AGB_SNAPSHOT_MAGIC;
    h.version = AGB_SNAPSHOT_VERSION;
    h.seed = w->d.seed;
    h.tick = w->tick;
    h.sim_time_s = w->sim_time;
    h.cell_count = st.count;
    h.cell_capacity = w->c.capacity;
    h.taumoeba_count = ts.count;
    h.taumoeba_capacity = w->tau_cap;
    h.n_temp = w->c.g[AGB_FIELD_TEMPERATURE].enabled ? w->c.g[AGB_FIELD_TEMPERATURE].nx : 0;
    h.n_co2 = w->c.g[AGB_FIELD_CO2].enabled ? w->c.g[AGB_FIELD_CO2].nx : 0;
    h.n_n2 = w->c.g[AGB_FIELD_N2].enabled ? w->c.g[AGB_FIELD_N2].nx : 0;
    h.chamber_w = w->d.chamber_w;
    h.chamber_h = w->d.chamber_h;
    h.chamber_d = w->d.chamber_d;
    h.physics_rate = w->physics_rate;
    h.biology_rate = w->biology_rate;
    h.next_cell_id = st.next_id;
    h.override_count = n_over;
    h.non_canon_run = n_over > 0 ? 1 : 0;
    if (scenario_id) std::strncpy(h.scenario_id, scenario_id, sizeof(h.scenario_id) - 1);
    std::strncpy(h.build_describe, "dev", sizeof(h.build_describe) - 1);
    h.state_hash = agb_fnv1a64(out + sizeof(h), (uint64_t)body, AGB_FNV1A64_OFFSET);
    std::memcpy(out, &h, sizeof(h));
    return AGB_OK;
}

agb_status agb_world_snapshot_load(const agb_world_desc* base, const void* data, int64_t n, agb_world** out) {
    if (!out) return AGB_INVALID_ARGUMENT;
    *out = nullptr;
    if (!base || !data || n < (int64_t)sizeof(agb_snapshot_header)) return AGB_FILE_IO_ERROR;
    agb_snapshot_header h;
    std::memcpy(&h, data, sizeof(h));
    if (h.magic != AGB_SNAPSHOT_MAGIC) return AGB_INVALID_ARGUMENT;
    if (h.version != AGB_SNAPSHOT_VERSION) return AGB_CONTRACT_VERSION_MISMATCH;
    const char* body = static_cast<const char*>(data) + sizeof(h);
    const uint64_t body_len = (uint64_t)(n - (int64_t)sizeof(h));
    if (agb_fnv1a64(body, body_len, AGB_FNV1A64_OFFSET) != h.state_hash) return AGB_INVALID_ARGUMENT;
    if (h.cell_count < 0 || h.cell_count > h.cell_capacity || h.override_count < 0) return AGB_INVALID_ARGUMENT;
    if (h.taumoeba_count < 0 || h.taumoeba_count > h.taumoeba_capacity) return AGB_INVALID_ARGUMENT;

    agb_world_desc d = *base;
    d.chamber_w = h.chamber_w;
    d.chamber_h = h.chamber_h;
    d.chamber_d = h.chamber_d;
    d.capacity = h.cell_capacity;
    d.tau_capacity = h.taumoeba_capacity;
    d.seed = h.seed;
    d.physics_rate = h.physics_rate;
    d.biology_rate = h.biology_rate;
    const int32_t want[3] = {h.n_temp, h.n_co2, h.n_n2};
    for (int k = 0; k < 3; ++k)
        if ((d.grid[kStoredFields[k]].nx > 0 ? d.grid[kStoredFields[k]].nx : 0) != want[k])
            return AGB_INVALID_ARGUMENT;                           // field resolution mismatch
    const char* cur = body;
    const char* end = body + body_len;
    double flash_power = AGB_PETROVA_FLASH_POWER;
    for (int32_t i = 0; i < h.override_count; ++i) {               // overrides come first
        if (cur + sizeof(agb_param_override) > end) return AGB_INVALID_ARGUMENT;
        agb_param_override ov;
        std::memcpy(&ov, cur, sizeof(ov));
        cur += sizeof(ov);
        if (std::strncmp(ov.key, "CO2_MASS_PER_DIVISION", sizeof(ov.key)) == 0) d.co2_mass_per_division = ov.value;
        if (std::strncmp(ov.key, "PETROVA_MAX_POWER", sizeof(ov.key)) == 0) d.max_emit_power = ov.value;
        if (std::strncmp(ov.key, "PETROVA_FLASH_POWER", sizeof(ov.key)) == 0) flash_power = ov.value;
    }
    agb_world* w = nullptr;
    agb_status rc = agb_world_create(&d, &w);
    if (rc != AGB_OK) return rc;
    w->flash_power = flash_power;                                   // the flash stays disarmed
    // Cells: the arrays are laid end to end; import takes one pointer per array.
    const size_t cnt = (size_t)h.cell_count;
    size_t need = 0;
    for (size_t e : kElem) need += e * cnt;
    if ((size_t)(end - cur) < need) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
    std::vector<char> cells(need ? need : 1);
    std::memcpy(cells.data(), cur, need);
    cur += need;
    void* p[25];
    {
        char* q = cells.data();
        for (int k = 0; k < 25; ++k) { p[k] = q; q += kElem[k] * cnt; }
    }
    agb_cells hc{(uint64_t*)p[0], (uint32_t*)p[1], (uint8_t*)p[2], (double*)p[3], (double*)p[4], (double*)p[5],
                 (double*)p[6], (double*)p[7], (double*)p[8], (double*)p[9], (float*)p[10], (float*)p[11],
                 (float*)p[12], (float*)p[13], (float*)p[14], (double*)p[15], (double*)p[16], (float*)p[17],
                 (uint64_t*)p[18], (float*)p[19], (float*)p[20], (float*)p[21], (float*)p[22], (float*)p[23],
                 (float*)p[24]};
    rc = agb_world_import_cells(w, &hc, h.cell_count, h.next_cell_id, nullptr);
    if (rc != AGB_OK) { agb_world_destroy(w); return rc; }
    // Predators: the header carries no next predator id and the reference's
    // loader leaves it at its initial value (snapshot.cu:218-219); so does this one.
    const size_t tcnt = (size_t)h.taumoeba_count;
    if (tcnt > 0) {
        size_t tneed = 0;
        for (size_t e : kTauElem) tneed += e * tcnt;
        if ((size_t)(end - cur) < tneed) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
        std::vector<char> tau(tneed);
        std::memcpy(tau.data(), cur, tneed);
        cur += tneed;
        void* t[20];
        char* q = tau.data();
        for (int k = 0; k < 20; ++k) { t[k] = q; q += kTauElem[k] * tcnt; }
        agb_taumoeba ht{(uint64_t*)t[0], (uint32_t*)t[1], (double*)t[2], (double*)t[3], (double*)t[4],
                        (double*)t[5], (double*)t[6], (double*)t[7], (float*)t[8], (float*)t[9], (float*)t[10],
                        (double*)t[11], (double*)t[12], (float*)t[13], (float*)t[14], (uint32_t*)t[15],
                        (uint64_t*)t[16], (float*)t[17], (float*)t[18], (int32_t*)t[19]};
        rc = agb_world_import_taumoeba(w, &ht, h.taumoeba_count, 1, nullptr);
        if (rc != AGB_OK) { agb_world_destroy(w); return rc; }
    }
    for (int f : kStoredFields) {
        const GridDev& g = w->c.g[f];
        if (!g.enabled) continue;
        const size_t bytes = 4 * (size_t)g.count;
        if ((size_t)(end - cur) < bytes) { agb_world_destroy(w); return AGB_INVALID_ARGUMENT; }
        std::vector<float> v((size_t)g.count);
        std::memcpy(v.data(), cur, bytes);
        cur += bytes;
        rc = agb_world_import_field(w, f, v.data(), nullptr);
        if (rc != AGB_OK) { agb_world_destroy(w); return rc; }
    }
    world_set_clock_state(w, h.tick, h.sim_time_s);
    *out = w;
    return AGB_OK;
}

}  // extern "C"
