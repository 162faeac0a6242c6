"""The World's between-tick knobs as the reference's callers set them: the store
charge (cell_store_set_charge, src/sim/cell_store.cu:281-297), a field's
boundary kind (Grid2D::bc, assigned by tests/physics/test_thermal.cu), the clock
rates assigned directly (read unclamped by src/sim/step.cu:133) and the live
overrides (World::co2_mass_per_division / petrova_max_power). Each is checked
against a world created with the same setting from the start, over eager and
graph-replayed ticks."""
import numpy as np
import pytest

import helpers as H

agb = H.agb
pytestmark = pytest.mark.gpu
CO2_SAT = 1.5          # CO2_SAT_CONC_1ATM [kg/m^3]: saturating, so cells take up CO2 and divide


def small_desc(**kw):
    d = agb.default_desc(capacity=kw.pop("capacity", 4000), co2_init=kw.pop("co2_init", 0.0))
    d.chamber_w = d.chamber_h = 1.0e-3
    d.grid[agb.FIELD_T] = agb.grid(64, 1, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT,
                                   agb.DEPOSIT_SCALE[0], kw.pop("t_bc", agb.BC_ROBIN))
    d.grid[agb.FIELD_CO2] = agb.grid(32, 1, agb.CO2_DIFFUSIVITY_WATER, d.grid[agb.FIELD_CO2].init,
                                     agb.DEPOSIT_SCALE[1], agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.grid(32, 1, agb.N2_DIFFUSIVITY, 0.0, agb.DEPOSIT_SCALE[2], agb.BC_NEUMANN)
    d.grid[agb.FIELD_IRR] = agb.grid(64, 1, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, agb.DEPOSIT_SCALE[3],
                                     agb.BC_NEUMANN)
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def populated(d, n=1500, awake=True, charge=0.5):
    w = agb.World(d)
    w.spawn(agb.spawn(n, charge_a=charge, awake=awake))
    return w


def assert_same(a, b):
    x, nx = a.export_cells()
    y, ny = b.export_cells()
    assert nx == ny and x.n == y.n
    for name, _t in agb.CELL_FIELDS:
        assert np.array_equal(x[name].view(np.uint8), y[name].view(np.uint8)), name
    for f in range(4):
        if a.desc.grid[f].nx > 0:
            assert np.array_equal(a.export_field(f).view(np.uint32), b.export_field(f).view(np.uint32)), f


def test_set_charge_sets_every_occupied_store_and_clamps():
    w = populated(small_desc(), awake=False)
    for q, want in ((0.3, 0.3), (1.7, 1.0), (-2.0, 0.0)):
        w.set_charge(q)
        c, _ = w.export_cells()
        occ = (c["flags"] & agb.FLAG_OCCUPIED) != 0
        assert occ.all()
        assert np.all(c["energy"][occ] == want * agb.CELL_ENERGY_MAX)
    w.close()


def test_set_charge_leaves_free_slots_alone():
    d = small_desc()
    w = populated(d, n=200, awake=False)
    c, nid = w.export_cells()
    c["flags"][::3] = 0                        # three in ten slots free
    c["energy"][::3] = 7.0
    w.import_cells(c, nid)
    w.set_charge(0.25)
    e, _ = w.export_cells()
    assert np.all(e["energy"][::3] == 7.0)
    rest = np.ones(e.n, bool)
    rest[::3] = False
    assert np.all(e["energy"][rest] == 0.25 * agb.CELL_ENERGY_MAX)
    w.close()


@pytest.mark.parametrize("graph", [False, True])
def test_set_boundary_before_first_tick_equals_created_with_it(graph):
    a = populated(small_desc(t_bc=agb.BC_ROBIN))
    b = populated(small_desc(t_bc=agb.BC_NEUMANN))
    face = [agb.AMBIENT_TEMP_DEFAULT] * 6
    a.set_boundary(agb.FIELD_T, [agb.BC_NEUMANN] * 6, face)
    for _ in range(6):
        a.step(1, graph=graph)
        b.step(1, graph=graph)
    assert_same(a, b)
    a.close()
    b.close()


def test_set_boundary_mid_run_reaches_replayed_graphs():
    """Graphs captured under the old faces are dropped: replay after the change
    equals eager ticks after the same change, and differs from a run that kept
    the old faces."""
    a, b, ctl = populated(small_desc()), populated(small_desc()), populated(small_desc())
    for _ in range(3):
        a.step(1, graph=True)
        b.step(1)
        ctl.step(1, graph=True)
    assert_same(a, b)
    dirichlet = [agb.BC_DIRICHLET] * 6
    face = [agb.AMBIENT_TEMP_DEFAULT - 5.0] * 6
    a.set_boundary(agb.FIELD_T, dirichlet, face)
    b.set_boundary(agb.FIELD_T, dirichlet, face)
    for _ in range(4):
        a.step(1, graph=True)
        b.step(1)
        ctl.step(1, graph=True)
    assert_same(a, b)
    ta, tc = a.export_field(agb.FIELD_T), ctl.export_field(agb.FIELD_T)
    edge = (ta - tc)[..., 0]                                  # the x- face column of every row
    assert float(edge.max()) < 0.0                            # the held faces pulled the edge down
    for w in (a, b, ctl):
        w.close()


def test_set_boundary_rejects_bad_arguments():
    w = populated(small_desc(), n=10)
    with pytest.raises(agb.AgbError):
        w.set_boundary(agb.FIELD_T, [3] * 6, [300.0] * 6)
    with pytest.raises(agb.AgbError):
        w.set_boundary(agb.FIELD_T, [agb.BC_DIRICHLET] * 6, [float("nan")] * 6)
    w.close()


def test_set_rates_is_unclamped_and_set_clock_clamps():
    """biology_rate 2e7 assigned directly runs at 2e7 (the reference's perf test
    does this); the clamped setter caps it at CLOCK_BIOLOGY_MAX."""
    d = small_desc(co2_init=CO2_SAT, contact_enabled=0, adhesion_enabled=0,
                   emission_enabled=0, taxis_enabled=0)
    direct = populated(d, awake=False)
    created = populated(small_desc(co2_init=CO2_SAT, contact_enabled=0, adhesion_enabled=0,
                                   emission_enabled=0, taxis_enabled=0, biology_rate=2.0e7), awake=False)
    clamped = populated(d, awake=False)
    direct.set_rates(1.0, 2.0e7)
    clamped.set_clock(1.0, 2.0e7)
    for w in (direct, created, clamped):
        w.step(1, graph=True)
    assert_same(direct, created)
    held_direct = direct.export_cells()[0]["co2_held"].mean()
    held_clamped = clamped.export_cells()[0]["co2_held"].mean()
    assert held_direct > 5.0 * held_clamped
    with pytest.raises(agb.AgbError):
        direct.set_rates(0.0, 1.0)
    for w in (direct, created, clamped):
        w.close()


def test_set_overrides_equal_created_with_them():
    # At 1e8 a cell banks about 3e-15 kg of CO2 a tick: the halved quota is met
    # after about four ticks, the canon one after about seven.
    base = dict(co2_init=CO2_SAT, contact_enabled=0, adhesion_enabled=0, biology_rate=1.0e8, capacity=16000)
    quota, pmax = 0.5 * agb.CO2_MASS_PER_DIVISION, 0.25 * agb.PETROVA_MAX_POWER
    a = populated(small_desc(**base), n=1000)
    b = populated(small_desc(co2_mass_per_division=quota, max_emit_power=pmax, **base), n=1000)
    a.set_overrides(quota, pmax)
    for _ in range(6):
        a.step(1, graph=True)
        b.step(1, graph=True)
    assert_same(a, b)
    a.close()
    b.close()


def test_set_overrides_mid_run_reach_replayed_graphs():
    # At 1e8 a cell banks about 3e-15 kg of CO2 a tick: the halved quota is met
    # after about four ticks, the canon one after about seven.
    base = dict(co2_init=CO2_SAT, contact_enabled=0, adhesion_enabled=0, biology_rate=1.0e8, capacity=16000)
    quota, pmax = 0.5 * agb.CO2_MASS_PER_DIVISION, 0.25 * agb.PETROVA_MAX_POWER
    a, b, ctl = (populated(small_desc(**base), n=1000) for _ in range(3))
    for w in (a, b, ctl):
        w.step(2, graph=True)
    a.set_overrides(quota, pmax)
    b.set_overrides(quota, pmax)
    for _ in range(8):
        a.step(1, graph=True)
        b.step(1)
        ctl.step(1, graph=True)
    assert_same(a, b)
    x, y = a.export_cells()[0], ctl.export_cells()[0]
    assert not np.array_equal(x["co2_held"], y["co2_held"]) or x.n != y.n   # the halved quota took effect
    for w in (a, b, ctl):
        w.close()


def test_mirror_equals_the_separate_reads():
    """agb_world_mirror (one synchronisation) returns what the separate calls
    return: count, capacity, next id, counters, predators, device pointers."""
    # At 3e8 a cell banks ~9e-15 kg of CO2 a tick: divisions from the third tick.
    d = small_desc(co2_init=CO2_SAT, contact_enabled=0, adhesion_enabled=0, biology_rate=3.0e8, capacity=16000)
    d.tau_capacity = 64
    w = populated(d, n=1000)
    w.spawn_taumoeba(20, 7)
    for _ in range(8):
        w.step(1, graph=True)
        m = w.mirror()
        cells, nid = w.export_cells()
        tau, tnid = w.export_taumoeba()
        c = w.counters()
        assert m["count"] == w.count() == cells.n
        assert m["capacity"] == 16000
        assert m["next_id"] == nid
        assert (m["divisions_this_window"], m["deaths_total"], m["dead_slots_prev"], m["error"]) == tuple(c)
        assert m["tau_count"] == tau.n == 20 and m["tau_next_id"] == tnid
        assert all(p for p in m["pointers"])
    assert w.count() > 1000                          # divisions happened, so next id moved
    w.close()
