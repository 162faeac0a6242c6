"""The scenario spine on the CPU: parsing the reference's scenario files and
synthetic ones, the loader's arithmetic (capacities, clock, horizon), the
acceptance fits, and -- where the reference is built here -- the whole spine
(parse, instantiate, drive, sample, measure) over the oracle against the
reference's own scenario code (src/sim/scenario.cpp, src/sim/accept.cpp) over
the reference's World: the same cells, fields and measured values, bit for bit."""
import ctypes as C
import glob
import json
import math
import os

import numpy as np
import pytest

import helpers as H
import scenarios as TSD

agb = H.agb
S = H.load_scenario()
SCEN_DIR = os.path.join(H.ROOT, "oracle", "_ref", "scenarios")
REF_SCENARIOS = sorted(glob.glob(os.path.join(SCEN_DIR, "*.json")))
needs_ref_files = pytest.mark.skipif(not REF_SCENARIOS, reason="reference scenario files not present")
needs_ref = pytest.mark.skipif(not (H.ref_available() and REF_SCENARIOS), reason="reference not built here")


def text_of(sid):
    with open(os.path.join(SCEN_DIR, sid + ".json")) as fh:
        return fh.read()


# A scenario of this suite's own: every stimulus the engine supports, short
# windows from t = 0 so a few dozen ticks cover them, and accept checks of
# each kind the engine measures.
DRIVEN = {
    "schema": 2, "id": "driven-test", "seed": 4242,
    "chamber": {"w": 0.004, "h": 0.004, "d": 6.0e-5, "boundary_x": "reflecting", "boundary_y": "absorbing"},
    "medium": {"temp_init": 300.0, "co2_init": 0.8, "n2_init": 0.05, "ambient_temp": 295.0,
               "store_disposition": "retain"},
    "light": {"ambient": 2.0, "sources": [{"dir_x": 0.0, "dir_y": 1.0, "irradiance": 5000.0}]},
    "populations": [
        {"kind": "astrophage", "count": 600, "placement": "gaussian", "place_radius": 6.0e-4,
         "charge": {"dist": "uniform", "a": 0.0, "b": 0.3}, "awake": True},
        {"kind": "astrophage", "count": 0},
        {"kind": "astrophage", "count": 300, "placement": "disc", "place_x": 5.0e-4, "place_radius": 3.0e-4,
         "charge": {"dist": "constant", "value": 0.9}}],
    "compaction": True,
    "clock": {"preset": "custom", "physics_rate": 2.0, "biology_rate": 5.0e4},
    "drive": [
        {"kind": "heat", "t0_s": 0.0, "t1_s": 0.03, "x": 1.0e-4, "y": -2.0e-4, "radius": 6.0e-4, "v0": 200.0, "v1": 50.0},
        {"kind": "chill", "t0_s": 0.01, "t1_s": 0.05, "x": -8.0e-4, "y": 3.0e-4, "radius": 4.0e-4, "value": 80.0},
        {"kind": "inject_co2", "t0_s": 0.0, "t1_s": 0.04, "radius": 0.0, "value": 5.0},
        {"kind": "inject_n2", "t0_s": 0.02, "t1_s": 0.06, "x": 0.0, "y": 0.0, "radius": 1.0e-3, "v0": 1.0, "v1": 3.0},
        {"kind": "set_light", "t0_s": 0.02, "t1_s": 0.05, "v0": 8000.0, "v1": 0.0},
        {"kind": "set_n2", "t0_s": 0.06, "t1_s": 0.07, "value": 0.125},
        {"kind": "seed_cells", "t0_s": 0.04, "t1_s": 0.0, "value": 1000.0},
        {"kind": "flash", "t0_s": 0.05, "t1_s": 0.07}],
    "objective": {"text": "exercise the driver", "accept": [
        {"metric": "awake_fraction", "op": ">=", "value": 0.0},
        {"metric": "medium_temp_mean", "op": "~=", "value": 295.0, "tol": 0.1},
        {"metric": "medium_temp_max", "op": ">", "value": 0.0},
        {"metric": "boil_event_count", "op": "==", "value": 0},
        {"metric": "population_live", "op": ">", "value": 0},
        {"metric": "population_dead", "op": ">=", "value": 0},
        {"metric": "mean_charge", "op": "<", "value": 1.0},
        {"metric": "total_energy_j", "op": ">", "value": 0.0},
        {"metric": "charge_depth_correlation", "op": "<=", "value": 1.0},
        {"metric": "charge_height_correlation", "op": ">=", "value": -1.0},
        {"metric": "doubling_time_s", "op": ">=", "value": 0.0},
        {"metric": "impulse_per_cycle", "op": "~=", "value": 1.0, "tol": 0.01}]},
}


def test_driven_scenario_parses():
    s = S.parse(json.dumps(DRIVEN))
    assert s.id == "driven-test" and s.seed == 4242
    assert s.boundary_y == agb.WALL_ABSORBING and s.store_disposition == agb.STORE_RETAIN
    assert [p.count for p in s.populations] == [600, 0, 300]
    assert s.populations[2].charge_a == 0.9 and s.populations[2].placement == agb.PLACE_DISC
    assert [d.kind for d in s.drive] == [S.HEAT, S.CHILL, S.INJECT_CO2, S.INJECT_N2, S.SET_LIGHT, S.SET_N2,
                                         S.SEED_CELLS, S.FLASH]
    assert s.drive[1].v0 == s.drive[1].v1 == 80.0
    assert s.clock == S.CUSTOM and S.clock_rates(s.clock, s.physics_rate, s.biology_rate) == (2.0, 5.0e4)
    assert S.unsupported(s) is None
    assert S.capacities(s) == (agb.DEFAULT_CELLS, agb.DEFAULT_TAUMOEBA)


@needs_ref_files
def test_reference_scenarios_parse():
    ids = {}
    for path in REF_SCENARIOS:
        s = S.load(path)
        ids[s.id] = s
        assert s.populations, s.id
    assert all(S.unsupported(s) is None for s in ids.values())
    assert S.capacities(ids["taumoeba"]) == (52096, 4352)
    no_n2 = {agb.FIELD_N2: agb.GridDesc()}
    assert S.unsupported(ids["taumoeba"], no_n2) and S.unsupported(ids["bloom"], no_n2) is None


def test_parse_defaults_comments_and_errors():
    s = S.parse('{ // a comment\n "id": "x", /* block */ "seed": "not a number",'
                ' "chamber": 3, "medium": {"gravity_axis": "z", "thermal_active": false},'
                ' "populations": [{"count": 12.9, "placement": "nowhere", "awake": 1}],'
                ' "id": "second id ignored", "note": "// not a comment"}')
    assert s.id == "x" and s.seed == 20260802
    assert s.chamber_w == agb.CHAMBER_W and s.gravity_axis == agb.GRAVITY_Z and s.thermal_active == 0
    assert s.populations[0].count == 12 and s.populations[0].placement == agb.PLACE_UNIFORM
    assert s.populations[0].awake == 0                      # a number is not a flag
    for bad in ('[1, 2]', '{"a": 1,}', 'not json',
                '{"drive": [{"kind": "levitate"}]}',
                '{"objective": {"accept": [{"metric": "happiness"}]}}'):
        with pytest.raises(S.ScenarioError):
            S.parse(bad)


def test_capacities_clock_and_horizon():
    s = S.Scenario(populations=[S.Population(count=30000), S.Population(kind=S.TAUMOEBA, count=100)])
    assert S.capacities(s) == (64096, 656)
    s = S.Scenario(populations=[S.Population(count=5_000_000)])
    assert S.capacities(s)[0] == agb.MAX_CELLS
    assert S.clock_rates(S.GENERATIONAL) == (0.5, 1.0e6)
    assert S.clock_rates(S.CUSTOM, 500.0, 0.1) == (agb.CLOCK_PHYSICS_MAX, agb.CLOCK_BIOLOGY_MIN)
    s = S.Scenario(accept=[S.Check("population_live", after_s=2.5)],
                   drive=[S.Stimulus(S.HEAT, t0_s=1.0, t1_s=3.25), S.Stimulus(S.HEAT, t0_s=4.0, t1_s=0.0)])
    assert S.horizon_ticks(s, 1.0) == 4000
    assert S.horizon_ticks(S.Scenario(run_duration_s=0.5), 10.0) == 50
    assert S.horizon_ticks(S.Scenario(), 1.0) == 60000


def test_accept_eval_and_fits():
    c = S.Check("total_energy_j", op="approx", value=100.0, tol=0.05)
    assert S.accept_eval(c, 104.9) and not S.accept_eval(c, 105.1)
    c.tol_absolute, c.tol = 1, 0.5
    assert S.accept_eval(c, 99.6) and not S.accept_eval(c, 99.4)
    assert S.accept_eval(S.Check("x", op="ne", value=1.0), 2.0)
    assert S._pearson([1.0, 2.0, 3.0], [2.0, 4.0, 6.0]) == pytest.approx(1.0)
    assert S._pearson([1.0, 1.0], [0.0, 1.0]) == 0.0
    agg = S.Aggregates()
    rate = math.log(2.0) / 0.5
    agg.t_series = [0.1 * k for k in range(30)]
    agg.n_series = [100.0 * math.exp(rate * t) for t in agg.t_series]
    assert S._doubling_time(agg, 10.0) == pytest.approx(5.0, rel=1e-9)


@needs_ref
@pytest.mark.parametrize("sid,ticks", [("first-light", 40), ("three-percent-line", 12), ("bloom", 40),
                                       ("komorov", 40), ("shadow-garden", 25), ("spin-drive-face", 60),
                                       ("taumoeba", 12)])
def test_spine_matches_reference_scenario_code(sid, ticks):
    text = text_of(sid)
    s = S.parse(text)
    dw = S.instantiate(s, make_world=H.OracleWorld)
    ok, res = S.run_assert(s, dw, ticks=ticks, graph=False)
    rw, measured = H.RefWorld.from_scenario(text, ticks, dw.desc)
    try:
        assert [r[1] for r in res] == measured
        a, na = dw.world.export_cells()
        b, nb = rw.export_cells()
        assert a.n == b.n and na == nb
        for name, _t in agb.CELL_FIELDS:
            assert np.array_equal(a[name].view(np.uint8), b[name].view(np.uint8)), name
        for f in range(4):
            assert np.array_equal(dw.world.export_field(f).ravel(), rw.export_field(f).ravel()), f
    finally:
        rw.close()


@needs_ref
def test_driven_scenario_matches_reference():
    text = json.dumps(DRIVEN)
    s = S.parse(text)
    ticks = 45
    dw = S.instantiate(s, make_world=H.OracleWorld)
    _ok, res = S.run_assert(s, dw, ticks=ticks, graph=False)
    rw, measured = H.RefWorld.from_scenario(text, ticks, dw.desc)
    try:
        assert [r[1] for r in res] == measured
        a, _ = dw.world.export_cells()
        b, _ = rw.export_cells()
        assert a.n == b.n == 1000, "the seed_cells top-up refilled the population"
        for name, _t in agb.CELL_FIELDS:
            assert np.array_equal(a[name].view(np.uint8), b[name].view(np.uint8)), name
        for f in range(4):
            assert np.array_equal(dw.world.export_field(f).ravel(), rw.export_field(f).ravel()), f
    finally:
        rw.close()


@needs_ref
def test_flash_matches_reference():
    """flash_step (src/sim/flash.cu): armed for 30 ticks then disarmed for 10,
    the oracle's cells and audit equal the reference's, bit for bit."""
    d = TSD.slab_desc(cap=900, light=(1.0, 0.0, 1e4, 0.0))
    d.taxis_enabled = 1
    sp = agb.spawn(800, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.004, awake=True)
    r, o = H.RefWorld(d), H.OracleWorld(d)
    try:
        r.spawn(sp)
        o.spawn(sp)
        for k in range(40):
            on = k < 30
            r.lib.ref_set_flash(r.h, int(on), 0.0)
            o.set_flash(on)
            r.step(1)
            o.step(1)
        a, _ = o.export_cells()
        b, _ = r.export_cells()
        for name, _t in agb.CELL_FIELDS:
            assert np.array_equal(a[name].view(np.uint8), b[name].view(np.uint8)), name
        ri, rd = C.c_double(), C.c_double()
        r.lib.ref_flash_audit(r.h, C.byref(ri), C.byref(rd))
        oi, od = o.flash_audit()
        assert (oi, od) == (ri.value, rd.value)
        assert od > 0.0 and abs(oi * agb.C_LIGHT / od - 1.0) < 1e-6
    finally:
        r.close()
