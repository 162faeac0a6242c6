// headless.cpp -- the command-line runner over the C ABI (no Python):
//
//   headless --scenario ID|PATH [--scenarios-dir DIR] [--assert] [--ticks N] [--csv PATH]
//   headless --assert-deterministic [--ticks N] [--seed S] [--cells N]
//
// The scenario mode is tools/headless.cpp:178-258 of the reference over
// src/sim/scenario.cpp (parse, capacities, instantiate, apply_drive) and
// src/sim/accept.cpp (aggregates, metrics, checks), driving an agb_world: the
// same rules as the Python spine (scenario.py) -- JSON with comments, unknown
// accept metrics and drive kinds rejected, unknown enum strings taking their
// defaults, the horizon from the objective's duration or the latest accept or
// drive time, at most 2,000 Stats samples. Exit status: 0 ACCEPT (or a run
// without --assert), 1 REJECT, 2 a scenario that does not parse or build, 3 a
// device error. The determinism mode runs one seeded world twice and requires
// equal state hashes (the reference's INV-8 gate).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "agb.h"
#include "agb_canon.h"

namespace {

// ---------------------------------------------------------------------------
// A small JSON reader: objects (first of a repeated key wins on lookup),
// arrays, strings with the standard escapes, numbers, true/false/null, and
// `//` and `/* */` comments between tokens.
// ---------------------------------------------------------------------------
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double n = 0.0;
    std::string s;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;

    const JVal* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double num(const char* key, double d) const {
        const JVal* v = get(key);
        return v && v->kind == Num ? v->n : d;
    }
    bool flag(const char* key, bool d) const {
        const JVal* v = get(key);
        return v && v->kind == Bool ? v->b : d;
    }
    std::string text(const char* key, const char* d) const {
        const JVal* v = get(key);
        return v && v->kind == Str ? v->s : std::string(d);
    }
    const JVal* object(const char* key) const {
        const JVal* v = get(key);
        return v && v->kind == Obj ? v : nullptr;
    }
    const std::vector<JVal>& array(const char* key) const {
        static const std::vector<JVal> empty;
        const JVal* v = get(key);
        return v && v->kind == Arr ? v->arr : empty;
    }
};

class JParser {
public:
    explicit JParser(const std::string& t) : t_(t) {}
    bool parse(JVal& out) {
        if (!value(out, 0)) return false;
        skip();
        return i_ == t_.size();
    }

private:
    const std::string& t_;
    size_t i_ = 0;

    void skip() {
        for (;;) {
            while (i_ < t_.size() && (t_[i_] == ' ' || t_[i_] == '\t' || t_[i_] == '\n' || t_[i_] == '\r')) ++i_;
            if (t_.compare(i_, 2, "//") == 0) {
                while (i_ < t_.size() && t_[i_] != '\n') ++i_;
            } else if (t_.compare(i_, 2, "/*") == 0) {
                const size_t e = t_.find("*/", i_ + 2);
                i_ = e == std::string::npos ? t_.size() : e + 2;
            } else {
                return;
            }
        }
    }
    bool lit(const char* w) {
        const size_t n = std::strlen(w);
        if (t_.compare(i_, n, w) != 0) return false;
        i_ += n;
        return true;
    }
    bool str(std::string& out) {
        if (i_ >= t_.size() || t_[i_] != '"') return false;
        ++i_;
        while (i_ < t_.size() && t_[i_] != '"') {
            char c = t_[i_++];
            if (c == '\\') {
                if (i_ >= t_.size()) return false;
                const char e = t_[i_++];
                switch (e) {
                    case 'n': c = '\n'; break;
                    case 't': c = '\t'; break;
                    case 'r': c = '\r'; break;
                    case 'b': c = '\b'; break;
                    case 'f': c = '\f'; break;
                    case 'u': {
                        if (i_ + 4 > t_.size()) return false;
                        const unsigned long cp = std::strtoul(t_.substr(i_, 4).c_str(), nullptr, 16);
                        i_ += 4;
                        c = cp < 0x80 ? (char)cp : '?';
                        break;
                    }
                    default: c = e; break;
                }
            }
            out.push_back(c);
        }
        if (i_ >= t_.size()) return false;
        ++i_;
        return true;
    }
    bool value(JVal& v, int depth) {
        if (depth > 64) return false;
        skip();
        if (i_ >= t_.size()) return false;
        const char c = t_[i_];
        if (c == '{') {
            v.kind = JVal::Obj;
            ++i_;
            skip();
            if (i_ < t_.size() && t_[i_] == '}') { ++i_; return true; }
            for (;;) {
                skip();
                std::string key;
                if (!str(key)) return false;
                skip();
                if (i_ >= t_.size() || t_[i_] != ':') return false;
                ++i_;
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.obj.emplace_back(std::move(key), std::move(child));
                skip();
                if (i_ < t_.size() && t_[i_] == ',') { ++i_; continue; }
                if (i_ < t_.size() && t_[i_] == '}') { ++i_; return true; }
                return false;
            }
        }
        if (c == '[') {
            v.kind = JVal::Arr;
            ++i_;
            skip();
            if (i_ < t_.size() && t_[i_] == ']') { ++i_; return true; }
            for (;;) {
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.arr.push_back(std::move(child));
                skip();
                if (i_ < t_.size() && t_[i_] == ',') { ++i_; continue; }
                if (i_ < t_.size() && t_[i_] == ']') { ++i_; return true; }
                return false;
            }
        }
        if (c == '"') { v.kind = JVal::Str; return str(v.s); }
        if (lit("true")) { v.kind = JVal::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = JVal::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = JVal::Null; return true; }
        const char* p = t_.c_str() + i_;
        char* end = nullptr;
        v.n = std::strtod(p, &end);
        if (end == p) return false;
        v.kind = JVal::Num;
        i_ += (size_t)(end - p);
        return true;
    }
};

// ---------------------------------------------------------------------------
// The scenario (contracts/scenario_v3.h) as the loader reads it
// ---------------------------------------------------------------------------
enum { ASTROPHAGE = 0, TAUMOEBA = 1 };
enum { REALTIME = 0, MOTION, METABOLIC, GENERATIONAL, CUSTOM };
enum { HEAT = 0, CHILL, INJECT_CO2, INJECT_N2, SET_LIGHT, SET_N2, SEED_CELLS, FLASH };
enum Op { EQ = 0, NE, LT, LE, GT, GE, APPROX };

const char* const kMetrics[] = {"awake_fraction", "medium_temp_mean", "medium_temp_max", "boil_event_count",
                                "population_live", "population_dead", "mean_charge", "total_energy_j",
                                "mean_tau_tolerance", "max_tau_tolerance", "charge_depth_correlation",
                                "charge_height_correlation", "rise_velocity_empty", "fall_velocity_full",
                                "doubling_time_s", "impulse_per_cycle"};
enum Metric { AWAKE_FRACTION = 0, MEDIUM_TEMP_MEAN, MEDIUM_TEMP_MAX, BOIL_EVENT_COUNT, POPULATION_LIVE,
              POPULATION_DEAD, MEAN_CHARGE, TOTAL_ENERGY_J, MEAN_TAU_TOLERANCE, MAX_TAU_TOLERANCE,
              CHARGE_DEPTH_CORRELATION, CHARGE_HEIGHT_CORRELATION, RISE_VELOCITY_EMPTY, FALL_VELOCITY_FULL,
              DOUBLING_TIME_S, IMPULSE_PER_CYCLE, METRIC_COUNT };

struct Population {
    int kind = ASTROPHAGE, count = 0, placement = AGB_PLACE_UNIFORM, dist = AGB_DIST_CONSTANT, awake = 0;
    double place_x = 0.0, place_y = 0.0, place_radius = 0.0, a = 0.0, b = 0.0;
};
struct Stimulus {
    int kind = HEAT;
    double t0 = 0.0, t1 = 0.0, x = 0.0, y = 0.0, radius = 0.0, v0 = 0.0, v1 = 0.0;
};
struct Check {
    int metric = 0, op = EQ, tol_absolute = 0;
    double value = 0.0, tol = 0.0, after_s = 0.0;
};
struct Scenario {
    std::string id;
    uint64_t seed = 20260802ull;
    double chamber_w = AGB_CHAMBER_W, chamber_h = AGB_CHAMBER_H, chamber_d = AGB_CHAMBER_D;
    int boundary_x = AGB_WALL_REFLECTING, boundary_y = AGB_WALL_REFLECTING;
    double temp_init = AGB_AMBIENT_TEMP_DEFAULT, co2_init = 0.0, n2_init = 0.0, ambient_temp = AGB_AMBIENT_TEMP_DEFAULT;
    int store_disposition = AGB_STORE_VOID, gravity_axis = AGB_GRAVITY_Y, thermal_active = 1;
    int compaction = 0, tau_compaction = 0;
    bool have_light = false;
    float light_dx = 1.0f, light_dy = 0.0f, light_irr = 0.0f, ambient_irr = 0.0f;
    std::vector<Population> pops;
    int clock = REALTIME;
    double physics_rate = 1.0, biology_rate = 1.0;
    std::vector<Stimulus> drive;
    std::vector<Check> accept;
    double run_duration_s = 0.0;
};

int pick(const std::string& s, std::initializer_list<std::pair<const char*, int>> m, int d) {
    for (const auto& kv : m)
        if (s == kv.first) return kv.second;
    return d;
}

// scenario_parse (src/sim/scenario.cpp:139-317). Returns false with a reason.
bool parse_scenario(const std::string& text, Scenario& s, std::string& why) {
    JVal root;
    if (!JParser(text).parse(root) || root.kind != JVal::Obj) { why = "scenario: not a JSON object"; return false; }
    s = Scenario{};
    s.id = root.text("id", "");
    s.seed = (uint64_t)(int64_t)root.num("seed", 20260802.0);
    if (const JVal* ch = root.object("chamber")) {
        s.chamber_w = ch->num("w", AGB_CHAMBER_W);
        s.chamber_h = ch->num("h", AGB_CHAMBER_H);
        s.chamber_d = ch->num("d", AGB_CHAMBER_D);
        s.boundary_x = pick(ch->text("boundary_x", "reflecting"), {{"periodic", AGB_WALL_PERIODIC}, {"absorbing", AGB_WALL_ABSORBING}}, AGB_WALL_REFLECTING);
        s.boundary_y = pick(ch->text("boundary_y", "reflecting"), {{"periodic", AGB_WALL_PERIODIC}, {"absorbing", AGB_WALL_ABSORBING}}, AGB_WALL_REFLECTING);
    }
    if (const JVal* md = root.object("medium")) {
        s.temp_init = md->num("temp_init", AGB_AMBIENT_TEMP_DEFAULT);
        s.co2_init = md->num("co2_init", 0.0);
        s.n2_init = md->num("n2_init", 0.0);
        s.ambient_temp = md->num("ambient_temp", AGB_AMBIENT_TEMP_DEFAULT);
        s.store_disposition = pick(md->text("store_disposition", "void"), {{"flash", AGB_STORE_FLASH}, {"retain", AGB_STORE_RETAIN}}, AGB_STORE_VOID);
        s.gravity_axis = md->text("gravity_axis", "y") == "z" ? AGB_GRAVITY_Z : AGB_GRAVITY_Y;
        s.thermal_active = md->flag("thermal_active", true) ? 1 : 0;
    }
    if (const JVal* lt = root.object("light")) {
        s.ambient_irr = (float)lt->num("ambient", 0.0);
        const auto& src = lt->array("sources");
        if (!src.empty()) {
            s.have_light = true;
            s.light_dx = (float)src[0].num("dir_x", 1.0);
            s.light_dy = (float)src[0].num("dir_y", 0.0);
            s.light_irr = (float)src[0].num("irradiance", 0.0);
        }
    }
    for (const JVal& p : root.array("populations")) {
        if (s.pops.size() >= 8) break;
        Population q;
        q.kind = p.text("kind", "astrophage") == "taumoeba" ? TAUMOEBA : ASTROPHAGE;
        q.count = (int)p.num("count", 0.0);
        q.placement = pick(p.text("placement", "uniform"), {{"gaussian", AGB_PLACE_GAUSSIAN}, {"grid", AGB_PLACE_GRID}, {"disc", AGB_PLACE_DISC}}, AGB_PLACE_UNIFORM);
        q.place_x = p.num("place_x", 0.0);
        q.place_y = p.num("place_y", 0.0);
        q.place_radius = p.num("place_radius", 0.0);
        if (const JVal* cg = p.get("charge")) {
            q.dist = pick(cg->text("dist", "constant"), {{"uniform", AGB_DIST_UNIFORM}, {"normal", AGB_DIST_NORMAL}}, AGB_DIST_CONSTANT);
            q.a = cg->num("value", cg->num("a", 0.0));
            q.b = cg->num("b", 0.0);
        }
        q.awake = p.flag("awake", false) ? 1 : 0;
        s.pops.push_back(q);
    }
    s.compaction = root.flag("compaction", false) ? 1 : 0;
    s.tau_compaction = root.flag("tau_compaction", false) ? 1 : 0;
    if (const JVal* ck = root.object("clock")) {
        s.clock = pick(ck->text("preset", "realtime"), {{"motion", MOTION}, {"metabolic", METABOLIC}, {"generational", GENERATIONAL}, {"custom", CUSTOM}}, REALTIME);
        s.physics_rate = ck->num("physics_rate", 1.0);
        s.biology_rate = ck->num("biology_rate", 1.0);
    }
    for (const JVal& e : root.array("drive")) {
        if (s.drive.size() >= 16) break;
        const int k = pick(e.text("kind", ""), {{"heat", HEAT}, {"chill", CHILL}, {"inject_co2", INJECT_CO2}, {"inject_n2", INJECT_N2},
                                               {"set_light", SET_LIGHT}, {"set_n2", SET_N2}, {"seed_cells", SEED_CELLS}, {"flash", FLASH}}, -1);
        if (k < 0) { why = "scenario: unknown drive stimulus kind"; return false; }
        Stimulus st;
        st.kind = k;
        st.t0 = e.num("t0_s", 0.0);
        st.t1 = e.num("t1_s", 0.0);
        st.x = e.num("x", 0.0);
        st.y = e.num("y", 0.0);
        st.radius = e.num("radius", 0.0);
        st.v0 = e.num("v0", e.num("value", 0.0));
        st.v1 = e.num("v1", e.num("value", st.v0));
        s.drive.push_back(st);
    }
    if (const JVal* ob = root.object("objective")) {
        s.run_duration_s = ob->num("duration_s", 0.0);
        for (const JVal& c : ob->array("accept")) {
            if (s.accept.size() >= 16) break;
            Check k;
            const std::string m = c.text("metric", "");
            k.metric = -1;
            for (int i = 0; i < METRIC_COUNT; ++i)
                if (m == kMetrics[i]) k.metric = i;
            if (k.metric < 0) { why = "scenario: unknown accept metric"; return false; }
            k.op = pick(c.text("op", "=="), {{"!=", NE}, {"<", LT}, {"<=", LE}, {">", GT}, {">=", GE}, {"~=", APPROX}}, EQ);
            k.value = c.num("value", 0.0);
            k.tol = c.num("tol", 0.0);
            k.after_s = c.num("after_s", 0.0);
            k.tol_absolute = c.flag("tol_absolute", false) ? 1 : 0;
            s.accept.push_back(k);
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// scenario_instantiate and scenario_apply_drive over an agb_world
// ---------------------------------------------------------------------------
void clock_rates(const Scenario& s, double& p, double& b) {   // world_set_clock, step.cu:190-215
    p = s.physics_rate;
    b = s.biology_rate;
    switch (s.clock) {
        case MOTION: p = AGB_CLOCK_MOTION_PHYSICS; b = AGB_CLOCK_MOTION_BIOLOGY; break;
        case METABOLIC: p = AGB_CLOCK_METABOLIC_PHYSICS; b = AGB_CLOCK_METABOLIC_BIOLOGY; break;
        case GENERATIONAL: p = AGB_CLOCK_GENERATIONAL_PHYSICS; b = AGB_CLOCK_GENERATIONAL_BIOLOGY; break;
        case CUSTOM: break;
        default: p = AGB_CLOCK_REALTIME_PHYSICS; b = AGB_CLOCK_REALTIME_BIOLOGY; break;
    }
    p = p < AGB_CLOCK_PHYSICS_MIN ? AGB_CLOCK_PHYSICS_MIN : (p > AGB_CLOCK_PHYSICS_MAX ? AGB_CLOCK_PHYSICS_MAX : p);
    b = b < AGB_CLOCK_BIOLOGY_MIN ? AGB_CLOCK_BIOLOGY_MIN : (b > AGB_CLOCK_BIOLOGY_MAX ? AGB_CLOCK_BIOLOGY_MAX : b);
}

struct Driven {
    agb_world* w = nullptr;
    agb_world_desc d{};
    agb_light light{};
    bool flash = false;
    uint64_t tick = 0;
    double sim_time = 0.0;
    ~Driven() { if (w) agb_world_destroy(w); }
    double dt() const { return AGB_DT_PHYSICS * d.physics_rate; }
    int64_t voxels(int f) const { return (int64_t)d.grid[f].nx * d.grid[f].ny * d.grid[f].nz; }
};

agb_spawn spawn_of(const Population& p, int32_t count) {
    agb_spawn sp{};
    sp.count = count;
    sp.placement = p.placement;
    sp.charge_dist = p.dist;
    sp.awake = p.awake;
    sp.place_x = p.place_x;
    sp.place_y = p.place_y;
    sp.place_radius = p.place_radius;
    sp.charge_a = p.a;
    sp.charge_b = p.b;
    return sp;
}

agb_status fill(Driven& dw, int f, double v) {
    std::vector<float> buf((size_t)dw.voxels(f), (float)v);
    return agb_world_import_field(dw.w, f, buf.data(), nullptr);
}

// scenario_capacities + scenario_instantiate (src/sim/scenario.cpp:325-397).
agb_status instantiate(const Scenario& s, Driven& dw) {
    int64_t cells = 0, tau = 0;
    for (const Population& p : s.pops) (p.kind == TAUMOEBA ? tau : cells) += p.count;
    int64_t cap = cells * 2 + 4096;
    cap = cap < AGB_DEFAULT_CELLS ? AGB_DEFAULT_CELLS : (cap > AGB_MAX_CELLS ? AGB_MAX_CELLS : cap);
    const int64_t tcap = tau * 4 + AGB_DEFAULT_TAUMOEBA;
    agb_world_desc& d = dw.d;
    agb_world_desc_default(&d);
    d.capacity = (int32_t)cap;
    d.tau_capacity = (int32_t)(tcap > AGB_MAX_TAUMOEBA ? AGB_MAX_TAUMOEBA : tcap);
    d.seed = s.seed;
    d.chamber_w = s.chamber_w; d.chamber_h = s.chamber_h; d.chamber_d = s.chamber_d;
    d.boundary_x = s.boundary_x; d.boundary_y = s.boundary_y;
    d.gravity_axis = s.gravity_axis;
    d.ambient_temp = s.ambient_temp;
    d.store_disposition = s.store_disposition;
    d.thermal_enabled = s.thermal_active ? 1 : 0;
    d.compaction_enabled = s.compaction ? 1 : 0;
    d.tau_compaction_enabled = s.tau_compaction ? 1 : 0;
    d.grid[AGB_FIELD_TEMPERATURE].init = s.ambient_temp;       // created at the ambient temperature
    d.grid[AGB_FIELD_CO2].init = s.co2_init;
    for (int k = 0; k < 6; ++k) {
        d.grid[AGB_FIELD_TEMPERATURE].face_value[k] = s.ambient_temp;
        d.grid[AGB_FIELD_CO2].face_value[k] = s.co2_init;
    }
    d.light.dir_x = 1.0f; d.light.dir_y = 0.0f; d.light.dir_z = 0.0f;
    d.light.irradiance = 0.0f; d.light.enabled = 0;
    if (s.have_light) {
        d.light.dir_x = s.light_dx; d.light.dir_y = s.light_dy;
        d.light.irradiance = s.light_irr; d.light.enabled = 1;
    }
    d.light.ambient = s.ambient_irr;
    clock_rates(s, d.physics_rate, d.biology_rate);
    dw.light = d.light;
    agb_status rc = agb_world_create(&d, &dw.w);
    if (rc) return rc;
    if (s.temp_init != s.ambient_temp && (rc = fill(dw, AGB_FIELD_TEMPERATURE, s.temp_init))) return rc;
    if (s.n2_init != 0.0 && (rc = fill(dw, AGB_FIELD_N2, s.n2_init))) return rc;
    uint64_t seed = s.seed;
    for (const Population& p : s.pops) {
        if (p.count <= 0) continue;
        if (p.kind == TAUMOEBA) rc = agb_world_spawn_taumoeba(dw.w, p.count, seed, nullptr);
        else {
            const agb_spawn sp = spawn_of(p, p.count);
            rc = agb_world_spawn_seeded(dw.w, &sp, seed, nullptr);
        }
        if (rc) return rc;
        ++seed;
    }
    return AGB_OK;
}

// scenario_apply_drive (src/sim/scenario.cpp:399-468) for the current tick.
agb_status apply_drive(const Scenario& s, Driven& dw) {
    const double t = dw.sim_time, dt = dw.dt();
    bool flash = false;
    for (const Stimulus& st : s.drive) {
        const bool open_ended = st.t1 <= st.t0;
        if (t < st.t0 || (!open_ended && t >= st.t1)) continue;
        const double frac = open_ended ? 0.0 : (t - st.t0) / (st.t1 - st.t0);
        const double strength = st.v0 + (st.v1 - st.v0) * frac;
        const double radius = st.radius > 0.0 ? st.radius : 10.0 * (s.chamber_w + s.chamber_h);
        agb_status rc = AGB_OK;
        switch (st.kind) {
            case HEAT: rc = agb_world_apply_brush(dw.w, AGB_BRUSH_HEAT, st.x, st.y, radius, strength * dt, nullptr); break;
            case CHILL: rc = agb_world_apply_brush(dw.w, AGB_BRUSH_CHILL, st.x, st.y, radius, strength * dt, nullptr); break;
            case INJECT_CO2: rc = agb_world_apply_brush(dw.w, AGB_BRUSH_INJECT_CO2, st.x, st.y, radius, strength * dt, nullptr); break;
            case INJECT_N2: rc = agb_world_apply_brush(dw.w, AGB_BRUSH_INJECT_N2, st.x, st.y, radius, strength * dt, nullptr); break;
            case SET_LIGHT: {
                const float irr = (float)strength;
                const int32_t on = strength > 0.0 ? 1 : 0;
                if (irr != dw.light.irradiance || on != dw.light.enabled) {
                    dw.light.irradiance = irr;
                    dw.light.enabled = on;
                    rc = agb_world_set_light(dw.w, &dw.light);
                }
                break;
            }
            case SET_N2: rc = fill(dw, AGB_FIELD_N2, strength); break;
            case SEED_CELLS: {
                int32_t count = 0;
                if ((rc = agb_world_count(dw.w, &count, nullptr))) break;
                const int32_t deficit = (int32_t)strength - count;
                for (const Population& p : s.pops) {
                    if (deficit <= 0) break;
                    if (p.kind != ASTROPHAGE) continue;
                    // cell_store_spawn refuses (and the driver ignores) a spawn past capacity.
                    if ((int64_t)count + deficit <= dw.d.capacity) {
                        const agb_spawn sp = spawn_of(p, deficit);
                        rc = agb_world_spawn_seeded(dw.w, &sp, s.seed + dw.tick, nullptr);
                    }
                    break;
                }
                break;
            }
            case FLASH: flash = true; break;
        }
        if (rc) return rc;
    }
    if (flash != dw.flash) {
        dw.flash = flash;
        return agb_world_set_flash(dw.w, flash ? 1 : 0, 0.0);
    }
    return AGB_OK;
}

// ---------------------------------------------------------------------------
// Acceptance (src/sim/accept.cpp)
// ---------------------------------------------------------------------------
double seqmean(const std::vector<double>& v) {
    double t = 0.0;
    for (double x : v) t += x;
    return t / (double)v.size();
}

double pearson(const std::vector<double>& a, const std::vector<double>& b) {
    const size_t n = a.size();
    if (n < 2 || b.size() != n) return 0.0;
    const double ma = seqmean(a), mb = seqmean(b);
    double sab = 0.0, saa = 0.0, sbb = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double da = a[i] - ma, db = b[i] - mb;
        sab += da * db;
        saa += da * da;
        sbb += db * db;
    }
    if (saa <= 0.0 || sbb <= 0.0) return 0.0;
    return sab / std::sqrt(saa * sbb);
}

struct Aggregates {
    int64_t boil_events = 0;
    double max_medium_k = 0.0;
    std::vector<double> t_series, n_series;
    int vel_stage = 0;
    double vel_ta = 0.0;
    std::vector<double> y_a, charge_a;
    double rise = 0.0, fall = 0.0;
};

// Positions (x, y) and energy of every slot, or false on a device error.
bool positions_energy(Driven& dw, std::vector<double>& x, std::vector<double>& y, std::vector<double>& e) {
    int32_t n = 0;
    if (agb_world_count(dw.w, &n, nullptr)) return false;
    x.assign((size_t)(n > 0 ? n : 1), 0.0);
    y.assign(x.size(), 0.0);
    e.assign(x.size(), 0.0);
    agb_cells c{};
    c.x = x.data(); c.y = y.data(); c.energy = e.data();
    int32_t cnt = 0;
    uint64_t nid = 0;
    if (agb_world_export_cells(dw.w, &c, n, &cnt, &nid, nullptr)) return false;
    const size_t m = (size_t)(cnt < n ? cnt : n);
    x.resize(m); y.resize(m); e.resize(m);
    return true;
}

bool aggregates_sample(Aggregates& a, const agb_stats& st, Driven& dw, bool velocity, bool population) {
    a.boil_events += st.boil_events;
    if (st.max_temp_medium_k > a.max_medium_k) a.max_medium_k = st.max_temp_medium_k;
    if (population) {
        a.t_series.push_back(st.sim_time_s);
        a.n_series.push_back((double)st.n_live);
    }
    if (!velocity) return true;
    const double settle_s = 2.0, interval_s = 4.0;
    std::vector<double> x, y, e;
    if (a.vel_stage == 0 && st.sim_time_s >= settle_s) {
        if (!positions_energy(dw, x, y, e)) return false;
        if (!y.empty()) {
            a.y_a = y;
            a.charge_a.resize(e.size());
            for (size_t i = 0; i < e.size(); ++i) a.charge_a[i] = e[i] / AGB_CELL_ENERGY_MAX;
            a.vel_ta = st.sim_time_s;
            a.vel_stage = 1;
        }
    } else if (a.vel_stage == 1 && st.sim_time_s >= a.vel_ta + interval_s) {
        if (!positions_energy(dw, x, y, e)) return false;
        if (y.empty()) return true;
        const double half_h = 0.5 * dw.d.chamber_h, margin = 3.0 * AGB_CELL_DIAMETER;
        const double dt = st.sim_time_s - a.vel_ta;
        const size_t m = y.size() < a.y_a.size() ? y.size() : a.y_a.size();
        std::vector<double> v, c;
        for (size_t i = 0; i < m; ++i) {
            if (std::fabs(y[i]) > half_h - margin) continue;
            v.push_back(-(y[i] - a.y_a[i]) / dt);
            c.push_back(a.charge_a[i]);
        }
        if (v.size() >= 2 && dt > 0.0) {
            const double mc = seqmean(c), mv = seqmean(v);
            double scv = 0.0, scc = 0.0;
            for (size_t i = 0; i < v.size(); ++i) {
                const double dc = c[i] - mc;
                scv += dc * (v[i] - mv);
                scc += dc * dc;
            }
            const double b = scc > 0.0 ? scv / scc : 0.0;
            a.rise = mv - b * mc;
            a.fall = a.rise + b;
        }
        a.vel_stage = 2;
    }
    return true;
}

double doubling_time(const Aggregates& a, double biology_rate) {
    if (a.n_series.size() < 2) return 0.0;
    double peak = 0.0;
    for (double n : a.n_series) peak = n > peak ? n : peak;
    if (peak <= 0.0) return 0.0;
    std::vector<double> t, l;
    for (size_t i = 0; i < a.n_series.size(); ++i)
        if (a.n_series[i] > 0.0 && a.n_series[i] <= 0.6 * peak) { t.push_back(a.t_series[i]); l.push_back(std::log(a.n_series[i])); }
    if (t.size() < 2) return 0.0;
    const double mt = seqmean(t), ml = seqmean(l);
    double stl = 0.0, stt = 0.0;
    for (size_t i = 0; i < t.size(); ++i) {
        const double d = t[i] - mt;
        stl += d * (l[i] - ml);
        stt += d * d;
    }
    if (stt <= 0.0) return 0.0;
    const double slope = stl / stt;
    return slope > 0.0 ? std::log(2.0) / slope * biology_rate : 0.0;
}

bool measure(int m, const agb_stats& fin, const Aggregates& a, Driven& dw, const Scenario& s, double& out) {
    std::vector<double> x, y, e;
    switch (m) {
        case AWAKE_FRACTION: out = fin.n_live > 0 ? (double)fin.n_awake / (double)fin.n_live : 0.0; return true;
        case MEDIUM_TEMP_MEAN: out = fin.mean_temp_medium_k; return true;
        case MEDIUM_TEMP_MAX: out = a.max_medium_k; return true;
        case BOIL_EVENT_COUNT: out = (double)a.boil_events; return true;
        case POPULATION_LIVE: out = (double)fin.n_live; return true;
        case POPULATION_DEAD: out = (double)fin.n_dead; return true;
        case MEAN_CHARGE: out = fin.mean_charge; return true;
        case TOTAL_ENERGY_J: out = fin.total_energy_j; return true;
        case MEAN_TAU_TOLERANCE: out = fin.mean_tau_tolerance; return true;
        case MAX_TAU_TOLERANCE: {
            agb_taumoeba t{};
            int32_t n = 0;
            uint64_t nid = 0;
            if (agb_world_export_taumoeba(dw.w, &t, 0, &n, &nid, nullptr)) return false;
            std::vector<uint32_t> fl((size_t)(n > 0 ? n : 1));
            std::vector<float> tol(fl.size());
            t.flags = fl.data();
            t.tolerance = tol.data();
            if (agb_world_export_taumoeba(dw.w, &t, n, &n, &nid, nullptr)) return false;
            out = 0.0;
            for (int32_t i = 0; i < n; ++i)
                if ((fl[i] & AGB_FLAG_OCCUPIED) && (fl[i] & AGB_FLAG_ALIVE) && (double)tol[i] > out) out = (double)tol[i];
            return true;
        }
        case CHARGE_DEPTH_CORRELATION:
        case CHARGE_HEIGHT_CORRELATION: {
            if (!positions_energy(dw, x, y, e)) return false;
            if (x.size() < 2) { out = 0.0; return true; }
            std::vector<double> c(e.size()), dep(e.size());
            for (size_t i = 0; i < e.size(); ++i) {
                c[i] = e[i] / AGB_CELL_ENERGY_MAX;
                dep[i] = x[i] * (double)s.light_dx + y[i] * (double)s.light_dy;
            }
            out = pearson(c, m == CHARGE_HEIGHT_CORRELATION ? y : dep);
            return true;
        }
        case RISE_VELOCITY_EMPTY: out = a.rise; return true;
        case FALL_VELOCITY_FULL: out = a.fall; return true;
        case DOUBLING_TIME_S: out = doubling_time(a, dw.d.biology_rate); return true;
        case IMPULSE_PER_CYCLE: {
            double imp = 0.0, dis = 0.0;
            if (agb_world_flash_audit(dw.w, &imp, &dis)) return false;
            out = dis > 0.0 ? imp * AGB_C_LIGHT / dis : 0.0;
            return true;
        }
    }
    return false;
}

bool accept_eval(const Check& c, double v) {   // accept_eval, accept.cpp:216-231
    switch (c.op) {
        case EQ: return v == c.value;
        case NE: return v != c.value;
        case LT: return v < c.value;
        case LE: return v <= c.value;
        case GT: return v > c.value;
        case GE: return v >= c.value;
        default: return std::fabs(v - c.value) <= (c.tol_absolute ? c.tol : c.tol * std::fabs(c.value));
    }
}

// ---------------------------------------------------------------------------
// The runner (tools/headless.cpp:178-258)
// ---------------------------------------------------------------------------
const char* op_symbol(int op) {
    static const char* sym[] = {"==", "!=", "<", "<=", ">", ">=", "~="};
    return sym[op];
}

int run_scenario(const Scenario& s, Driven& dw, bool do_assert, int64_t ticks_override, const char* csv_path) {
    if (do_assert && s.accept.empty()) {
        std::printf("scenario %s: no objective (sandbox) -- ACCEPT\n", s.id.c_str());
        return 0;
    }
    double horizon = s.run_duration_s;
    if (horizon <= 0.0) {
        for (const Check& c : s.accept) horizon = c.after_s > horizon ? c.after_s : horizon;
        for (const Stimulus& d : s.drive) {
            const double te = d.t1 > d.t0 ? d.t1 : d.t0;
            horizon = te > horizon ? te : horizon;
        }
    }
    if (horizon <= 0.0) horizon = 60.0;
    int64_t ticks = ticks_override > 0 ? ticks_override : (int64_t)std::ceil(horizon / dw.dt());
    if (ticks < 1) ticks = 1;
    const int64_t stride = ticks > 2000 ? ticks / 2000 : 1;
    bool velocity = false, population = false;
    for (const Check& c : s.accept) {
        velocity = velocity || c.metric == RISE_VELOCITY_EMPTY || c.metric == FALL_VELOCITY_FULL;
        population = population || c.metric == DOUBLING_TIME_S;
    }
    Aggregates agg;
    agb_stats st{};
    std::FILE* csv = csv_path ? std::fopen(csv_path, "w") : nullptr;
    if (csv) std::fprintf(csv, "# scenario: %s\n# seed: %llu\nt_s,n_live,n_dead,n_tau,mean_charge,total_energy_J,"
                               "mean_temp_cell_K,mean_temp_medium_K,co2_total_kg,mean_tolerance,boil_events,divisions,deaths\n",
                          s.id.c_str(), (unsigned long long)s.seed);
    auto row = [&](const agb_stats& r) {
        if (csv) std::fprintf(csv, "%.6f,%d,%d,%d,%.6f,%.6e,%.4f,%.4f,%.6e,%.6f,%d,%d,%d\n", r.sim_time_s, r.n_live,
                              r.n_dead, r.n_taumoeba, r.mean_charge, r.total_energy_j, r.mean_temp_cell_k,
                              r.mean_temp_medium_k, r.co2_total_kg, r.mean_tau_tolerance, r.boil_events,
                              r.divisions_this_window, r.deaths_this_window);
    };
    bool ok = true;
    for (int64_t t = 0; t < ticks && ok; ++t) {
        ok = apply_drive(s, dw) == AGB_OK && agb_world_step_graph(dw.w, 1, nullptr) == AGB_OK;
        ++dw.tick;
        dw.sim_time += dw.dt();
        if (ok && do_assert && t % stride == 0) {
            ok = agb_world_stats(dw.w, &st, nullptr) == AGB_OK && aggregates_sample(agg, st, dw, velocity, population);
            row(st);
        }
    }
    if (ok) ok = agb_world_stats(dw.w, &st, nullptr) == AGB_OK;
    if (ok && do_assert) ok = aggregates_sample(agg, st, dw, velocity, population);
    row(st);
    if (csv) std::fclose(csv);
    if (!ok) {
        std::printf("scenario %s: device error: %s\n", s.id.c_str(), agb_last_error(dw.w));
        return 3;
    }
    if (!do_assert) {
        std::printf("scenario %s: %lld ticks, %.3f s, live %d, dead %d, awake %d\n", s.id.c_str(), (long long)ticks,
                    st.sim_time_s, st.n_live, st.n_dead, st.n_awake);
        return 0;
    }
    std::printf("scenario %s: assert over %.1f s (%lld ticks, %d checks)\n", s.id.c_str(), st.sim_time_s,
                (long long)ticks, (int)s.accept.size());
    bool all = true;
    for (const Check& c : s.accept) {
        double v = 0.0;
        if (!measure(c.metric, st, agg, dw, s, v)) {
            std::printf("scenario %s: device error: %s\n", s.id.c_str(), agb_last_error(dw.w));
            return 3;
        }
        const bool pass = accept_eval(c, v);
        all = all && pass;
        std::printf("  [%s] %-26s %-12.6g %s %-.6g", pass ? "PASS" : "FAIL", kMetrics[c.metric], v, op_symbol(c.op),
                    c.value);
        if (c.op == APPROX) std::printf(" (tol %.4g%s)", c.tol, c.tol_absolute ? " abs" : " rel");
        if (c.after_s > 0.0) std::printf(" [after %.0f s]", c.after_s);
        std::printf("\n");
    }
    std::printf("scenario %s: %s\n", s.id.c_str(), all ? "ACCEPT" : "REJECT");
    return all ? 0 : 1;
}

// --assert-deterministic: one seeded world run twice; the state hashes must agree.
int run_deterministic(int64_t ticks, uint64_t seed, int32_t cells) {
    uint64_t h[2] = {0, 0};
    for (int r = 0; r < 2; ++r) {
        agb_world_desc d;
        agb_world_desc_default(&d);
        d.seed = seed;
        d.capacity = 2 * cells + 4096;
        agb_world* w = nullptr;
        if (agb_world_create(&d, &w) != AGB_OK) { std::printf("world_create failed\n"); return 3; }
        agb_spawn sp{};
        sp.count = cells;
        sp.charge_dist = AGB_DIST_CONSTANT;
        sp.charge_a = 0.02;
        sp.awake = 1;
        const bool ok = agb_world_spawn(w, &sp, nullptr) == AGB_OK && agb_world_step_graph(w, (int32_t)ticks, nullptr) == AGB_OK &&
                        agb_world_state_hash(w, &h[r], nullptr) == AGB_OK;
        if (!ok) { std::printf("device error: %s\n", agb_last_error(w)); agb_world_destroy(w); return 3; }
        agb_world_destroy(w);
    }
    std::printf("deterministic: %016llx %016llx %s\n", (unsigned long long)h[0], (unsigned long long)h[1],
                h[0] == h[1] ? "MATCH" : "MISMATCH");
    return h[0] == h[1] ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
    const char* scenario = nullptr;
    std::string dir = "scenarios";
    const char* csv = nullptr;
    bool do_assert = false, deterministic = false;
    int64_t ticks = 0;
    uint64_t seed = 20260802ull;
    int32_t cells = 4096;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : ""; };
        if (a == "--scenario") scenario = next();
        else if (a == "--scenarios-dir") dir = next();
        else if (a == "--assert") do_assert = true;
        else if (a == "--assert-deterministic") deterministic = true;
        else if (a == "--ticks") ticks = std::atoll(next());
        else if (a == "--seed") seed = std::strtoull(next(), nullptr, 10);
        else if (a == "--cells") cells = std::atoi(next());
        else if (a == "--csv") csv = next();
        else {
            std::printf("usage: headless --scenario ID|PATH [--scenarios-dir DIR] [--assert] [--ticks N] [--csv PATH]\n"
                        "       headless --assert-deterministic [--ticks N] [--seed S] [--cells N]\n");
            return a == "--help" || a == "-h" ? 0 : 2;
        }
    }
    if (deterministic) return run_deterministic(ticks > 0 ? ticks : 1000, seed, cells);
    if (!scenario) { std::printf("headless: --scenario or --assert-deterministic\n"); return 2; }
    std::string path = scenario;
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        path = dir + "/" + scenario + ".json";
        f = std::fopen(path.c_str(), "rb");
    }
    if (!f) { std::printf("scenario: cannot open file\n"); return 2; }
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    Scenario s;
    std::string why;
    if (!parse_scenario(text, s, why)) { std::printf("%s\n", why.c_str()); return 2; }
    Driven dw;
    const agb_status rc = instantiate(s, dw);
    if (rc != AGB_OK) {
        std::printf("scenario %s: cannot build the world: %s\n", s.id.c_str(), agb_status_str(rc));
        return 2;
    }
    return run_scenario(s, dw, do_assert, ticks, csv);
}
