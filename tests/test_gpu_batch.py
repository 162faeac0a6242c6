"""Batched ensembles: every chamber of a batch advanced by one graph launch per
step equals, bit for bit, a standalone world built from the same descriptor
(with the hash cell size the autotuner picked) and stepped tick by tick."""
import numpy as np
import pytest

import helpers as H

agb = H.agb
pytestmark = pytest.mark.gpu

EMAX = agb.CELL_ENERGY_MAX


def cube_desc(edge, cap, seed, span=1.0e-3, compaction=1, light_axis=2):
    d = agb.default_desc(capacity=cap, seed=seed, co2_init=1.0)
    d.chamber_w = d.chamber_h = d.chamber_d = span
    bc_t = [agb.BC_DIRICHLET] + [agb.BC_ROBIN] * 5
    face = [330.0] + [agb.AMBIENT_TEMP_DEFAULT] * 5
    d.grid[agb.FIELD_T] = agb.grid(edge, edge, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9,
                                   bc_t, face_value=face)
    d.grid[agb.FIELD_CO2] = agb.grid(edge, edge, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.GridDesc()
    d.grid[agb.FIELD_IRR] = agb.grid(edge, edge, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
    d.taxis_enabled = 0
    dirs = {0: (1.0, 0.0, 0.0), 1: (0.0, 1.0, 0.0), 2: (0.0, 0.0, 1.0)}[light_axis]
    d.light = agb.Light(dirs[0], dirs[1], dirs[2], 1.0e4, 0.0, 1)
    d.division_predicate = agb.DIVIDE_ENERGY
    d.division_energy = 0.16 * EMAX
    d.compaction_enabled = compaction
    d.compaction_period = 3
    d.biology_rate = 1.0e5
    return d


def chambers():
    """Four chambers of uneven grids, populations, seeds, charge and light."""
    spec = [(32, 400, 0.05, 2), (48, 2500, 0.12, 0), (40, 1200, 0.20, 1), (64, 6000, 0.08, 2)]
    descs, spawns = [], []
    for i, (edge, cells, q, axis) in enumerate(spec):
        descs.append(cube_desc(edge, 2 * cells, seed=11 + i, light_axis=axis))
        spawns.append(agb.spawn(cells, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=q, awake=True))
    return descs, spawns


def standalone(desc, sp, ticks, hash_cell=None, walk=None):
    """A world on its own, with the chamber's hash cell and walk shape (lanes
    per cell, fused): the same launch shape gives the same bits."""
    if hash_cell is not None:
        desc.hash_cell_size = hash_cell
    w = agb.World(desc)
    if walk is not None:
        w.walk(*walk)
    w.spawn(sp)
    w.step(ticks)
    return w


def assert_same(chamber, world, where):
    a, na = chamber.export_cells()
    b, nb = world.export_cells()
    assert na == nb and a.n == b.n, where
    for name, _t in agb.CELL_FIELDS:
        assert np.array_equal(a[name].view(np.uint8), b[name].view(np.uint8)), "%s: %s" % (where, name)
    for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2, agb.FIELD_IRR):
        if world.desc.grid[f].nx <= 0:
            continue
        assert np.array_equal(chamber.export_field(f).view(np.uint32), world.export_field(f).view(np.uint32)), \
            "%s: field %d" % (where, f)
    assert chamber.counters()[3] == 0 and world.counters()[3] == 0


@pytest.mark.parametrize("staged", [True, False])
def test_batch_equals_standalone_worlds(staged):
    descs, spawns = chambers()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=3, staged=staged))
    assert b.staged() == staged
    ticks = [1, 2, 1, 3, 1]                # mixed step sizes cross the compaction period
    for t in ticks:
        b.step(t)
    total = sum(ticks)
    for i in range(b.n):
        t = b.tuning(i)
        assert 0 <= t.lane < 3
        d, s = chambers()
        w = standalone(d[i], s[i], total, walk=b.chambers[i].walk())
        assert_same(b.chambers[i], w, "chamber %d" % i)
    assert b.graph_kernels() > 0


@pytest.mark.parametrize("staged", [True, False])
def test_batch_graph_replay_repeats(staged):
    """Stepping one tick at a time replays cached graphs; results still match."""
    descs, spawns = chambers()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=staged))
    assert b.staged() == staged
    for _ in range(8):
        b.step(1)
    k1 = b.graph_kernels()
    d, s = chambers()
    for i in range(b.n):
        w = standalone(d[i], s[i], 8, walk=b.chambers[i].walk())
        assert_same(b.chambers[i], w, "chamber %d" % i)
    b.step(1)
    assert b.graph_kernels() > k1


def test_autotuned_batch_matches_tuned_standalone():
    descs, spawns = chambers()
    cands = (1.0e-5, 1.6e-5, 2.2e-5)
    b = agb.Batch(descs, spawns, agb.batch_opts(autotune=True, hash_candidates=cands, probe_ticks=2))
    b.step(2)
    b.step(2)
    for i in range(b.n):
        t = b.tuning(i)
        assert any(abs(t.hash_cell_size - c) < 1e-12 for c in cands), t.as_dict()
        assert t.probe_tick_ms > 0.0
        assert t.ftcs_lx[0] in (16, 32) and t.ftcs_rpt[0] in (1, 2, 4) and t.ftcs_zc[0] >= 1
        d, s = chambers()
        w = standalone(d[i], s[i], 4, hash_cell=t.hash_cell_size, walk=b.chambers[i].walk())
        assert_same(b.chambers[i], w, "tuned chamber %d" % i)


def test_batch_stats_per_chamber():
    descs, spawns = chambers()
    b = agb.Batch(descs, spawns)
    b.step(2)
    st = b.stats()
    assert len(st) == b.n
    for i, s in enumerate(st):
        assert s.tick == 2
        assert s.n_live + s.n_dead == b.chambers[i].count()


@pytest.mark.parametrize("staged", [True, False])
def test_batch_with_n2_and_taxis(staged):
    """Chambers with an N2 grid (a second slow field) and taxis on (run and
    tumble inside the per-cell pass) equal their standalone worlds."""
    def make():
        descs, spawns = chambers()
        for d in descs:
            e = d.grid[agb.FIELD_T].nx
            d.grid[agb.FIELD_N2] = agb.grid(e, e, agb.N2_DIFFUSIVITY, 0.2, 1e15, agb.BC_NEUMANN)
            d.taxis_enabled = 1
        return descs, spawns
    descs, spawns = make()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=staged))
    assert b.staged() == staged
    for t in (2, 1, 2):
        b.step(t)
    for i in range(b.n):
        d, s = make()
        w = standalone(d[i], s[i], 5, walk=b.chambers[i].walk())
        assert_same(b.chambers[i], w, "chamber %d" % i)
