"""The engine against the oracle on the 3-D workloads the benchmark times.

cube2k (+z light, a Dirichlet x- face, 64^3 grids, 10 um buckets), slab25k
(+x light, the 550 um slab placement, lognormal charge, division at a
stored-energy threshold, compaction every 10 ticks, 128^3 grids) and
clusters20k (the 1M-cell cluster workload at 20,000 cells and 64^3 grids,
same core density, +z light, CO2-quota division, compaction every tick),
built by the same workload code the benchmark uses, from identical imported
state:

  * stage by stage for two ticks: every stage from the oracle's state after
    the previous one; hash keys, sorted order and bucket ranges bit-exact;
    cells, fields and forces within the parity bounds (parity.py);
  * 60 whole ticks, each from the oracle's state after the previous tick
    (graph-replayed ticks, the benchmark's path): integer state, the hash and
    the exact-zero irradiance set bit-exact, every floating-point cell value
    and field within the bounds, Stats counts equal -- across six compaction
    periods of slab25k;
  * 60 whole ticks free-running: integer state and Stats counts still equal,
    positions, energies and fields within 1e-5.

The batched ensemble's chambers (3-D grids, light along each axis, staged and
lane launches) are compared with the oracle the same way.
"""
import os

import numpy as np
import pytest

import helpers as H
import parity as P
import scenarios as S

agb = H.agb
W = H.load_workloads()
pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
TICKS = 60
# (workload, walk shape): the default shape of each workload, and the
# separate one-lane walks the 1M-cell workload runs with.
CASES = [("cube2k", None), ("slab25k", None), ("clusters20k", None), ("clusters20k", (1, False))]


def seeded(name, walk=None):
    d, sp, _ = W.workload(name, seed=1)
    orc = H.OracleWorld(d, threads=THREADS)
    orc.spawn(sp)
    gpu = agb.World(d)
    if walk is not None:
        assert gpu.walk(*walk) == walk
    P.copy_state(orc, gpu)
    return d, gpu, orc


def hash_errors(gpu, orc, where):
    errs = []
    for k, (x, y) in enumerate(zip(gpu.export_hash(), orc.export_hash())):
        if not np.array_equal(x, y):
            errs.append("%s: hash array %d differs" % (where, k))
    return errs


def stats_errors(gpu, orc, where, out=None):
    """Stats of both (each call closes the reporting window on both sides)."""
    sg, so = gpu.stats(), orc.stats()
    if out is not None:
        out.append(so)
    errs = []
    for k in ("tick", "n_live", "n_dead", "n_dormant", "n_awake", "divisions_this_window", "deaths_this_window",
              "boil_events", "ignitions_this_window"):
        if getattr(sg, k) != getattr(so, k):
            errs.append("%s: Stats.%s %s != %s" % (where, k, getattr(sg, k), getattr(so, k)))
    if abs(sg.total_energy_j - so.total_energy_j) > P.RTOL * abs(so.total_energy_j):
        errs.append("%s: total energy %.9e != %.9e" % (where, sg.total_energy_j, so.total_energy_j))
    return errs


@pytest.mark.parametrize("name,walk", CASES)
def test_3d_stage_by_stage(name, walk):
    d, gpu, orc = seeded(name, walk)
    src = P.source_irradiance(d)
    errs = []
    for t in range(2):
        for stage, sname in S.stages_for(d):
            P.copy_state(orc, gpu)
            if stage in (agb.STAGE_EMISSION, agb.STAGE_MOTION):
                gpu.stage(agb.STAGE_HASH)      # the tick's hash, rebuilt from unmoved positions
            gpu.stage(stage)
            orc.stage(stage)
            where = "tick %d %s" % (t, sname)
            if stage in (agb.STAGE_HASH, agb.STAGE_EMISSION, agb.STAGE_MOTION):
                errs += hash_errors(gpu, orc, where)
            a, _ = gpu.export_cells()
            b, _ = orc.export_cells()
            scales = orc.export_term_scales() if stage == agb.STAGE_MOTION else None
            errs += P.compare_cells(a, b, where=where, scales=scales, source=src)
            errs += P.compare_fields(gpu, orc, where=where)
            if stage == agb.STAGE_MOTION:
                errs += P.compare_forces(gpu.export_forces(), orc.export_forces(), where, scale=scales[0])
    assert gpu.counters()[3] == 0
    assert not errs, "\n".join(errs[:20])


@pytest.mark.parametrize("name,walk", CASES)
def test_3d_resynced_ticks(name, walk):
    d, gpu, orc = seeded(name, walk)
    src = P.source_irradiance(d)
    errs = []
    births = 0
    for t in range(TICKS):
        P.copy_state(orc, gpu)
        gpu.step(1, graph=True)
        orc.step(1)
        where = "tick %d" % t
        errs += hash_errors(gpu, orc, where)
        a, _ = gpu.export_cells()
        b, _ = orc.export_cells()
        errs += P.compare_cells(a, b, where=where, scales=orc.export_term_scales(), source=src)
        errs += P.compare_fields(gpu, orc, where=where)
        got = []
        errs += stats_errors(gpu, orc, where, got)
        births += got[0].divisions_this_window
        if len(errs) > 40:
            break
    assert gpu.counters()[3] == 0
    assert not errs, "\n".join(errs[:20])
    if name == "slab25k":
        # The run must exercise what it claims: divisions at the energy threshold.
        assert births > 0, "no divisions in %d ticks" % TICKS


@pytest.mark.parametrize("name", ["cube2k", "slab25k", "clusters20k"])
def test_3d_free_run(name):
    d, gpu, orc = seeded(name)
    src = P.source_irradiance(d)
    done = 0
    for t in (1, 10, 11, 30, TICKS):
        gpu.step(t - done, graph=True)
        orc.step(t - done)
        done = t
        a, _ = gpu.export_cells()
        b, _ = orc.export_cells()
        where = "after %d ticks" % t
        errs = P.compare_cells(a, b, where=where, source=src, velocities=False)
        # Free-running fields and per-cell samples inherit the positions' drift;
        # irradiance and samples are compared through the fields and positions.
        errs = [e for e in errs if not any(k in e for k in ("irradiance out", "t_local", "co2_local", "n2_local"))]
        errs += P.compare_fields(gpu, orc, where=where)
        errs += stats_errors(gpu, orc, where)
        assert not errs, "\n".join(errs[:20])
    assert gpu.counters()[3] == 0


# ---------------------------------------------------------------------------
# Batched chambers against the oracle
# ---------------------------------------------------------------------------
def batch_chambers():
    """Four 3-D chambers: uneven grids and populations, light along z, x, y, z,
    energy-threshold division with compaction every third tick."""
    spec = [(32, 400, 0.05, 2), (48, 2500, 0.12, 0), (40, 1200, 0.20, 1), (64, 6000, 0.08, 2)]
    descs, spawns = [], []
    for i, (edge, cells, q, axis) in enumerate(spec):
        d = agb.default_desc(capacity=2 * cells, seed=11 + i, co2_init=1.0)
        d.chamber_w = d.chamber_h = d.chamber_d = 1.0e-3
        d.grid[agb.FIELD_T] = agb.grid(edge, edge, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9,
                                       [agb.BC_DIRICHLET] + [agb.BC_ROBIN] * 5,
                                       face_value=[330.0] + [agb.AMBIENT_TEMP_DEFAULT] * 5)
        d.grid[agb.FIELD_CO2] = agb.grid(edge, edge, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
        d.grid[agb.FIELD_N2] = agb.GridDesc()
        d.grid[agb.FIELD_IRR] = agb.grid(edge, edge, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
        d.taxis_enabled = 0
        dirs = {0: (1.0, 0.0, 0.0), 1: (0.0, 1.0, 0.0), 2: (0.0, 0.0, 1.0)}[axis]
        d.light = agb.Light(dirs[0], dirs[1], dirs[2], 1.0e4, 0.0, 1)
        d.division_predicate = agb.DIVIDE_ENERGY
        d.division_energy = 0.16 * agb.CELL_ENERGY_MAX
        d.compaction_enabled = 1
        d.compaction_period = 3
        d.biology_rate = 1.0e5
        descs.append(d)
        spawns.append(agb.spawn(cells, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=q, awake=True))
    return descs, spawns


def chamber_oracles(b):
    """An oracle world per chamber, from the chamber's descriptor (with the hash
    cell the batch runs it with) and its state before the first step."""
    out = []
    for i in range(b.n):
        d = agb.WorldDesc.from_buffer_copy(b.descs[i])
        d.hash_cell_size = b.tuning(i).hash_cell_size
        orc = H.OracleWorld(d, threads=THREADS)
        P.copy_state(b.chambers[i], orc)
        out.append(orc)
    return out


@pytest.mark.parametrize("staged", [True, False])
def test_batch_chambers_track_oracle(staged):
    descs, spawns = batch_chambers()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=staged))
    assert b.staged() == staged
    orcs = chamber_oracles(b)
    errs = []
    # Resynchronised: every chamber from its oracle's state, one batched step.
    for t in range(12):
        for i in range(b.n):
            P.copy_state(orcs[i], b.chambers[i])
        b.step(1)
        for i, orc in enumerate(orcs):
            orc.step(1)
            where = "chamber %d tick %d" % (i, t)
            a, _ = b.chambers[i].export_cells()
            c, _ = orc.export_cells()
            errs += P.compare_cells(a, c, where=where, scales=orc.export_term_scales(),
                                    source=P.source_irradiance(orc.desc))
            errs += P.compare_fields(b.chambers[i], orc, where=where)
            errs += hash_errors(b.chambers[i], orc, where)
    # Free-running: integer state stays equal.
    b.step(9)
    for i, orc in enumerate(orcs):
        orc.step(9)
        a, _ = b.chambers[i].export_cells()
        c, _ = orc.export_cells()
        if a.n != c.n:
            errs.append("chamber %d free run: count %d != %d" % (i, a.n, c.n))
            continue
        for k in P.INT_FIELDS:
            if not np.array_equal(a[k], c[k]):
                errs.append("chamber %d free run: %s differs" % (i, k))
        errs += [e for e in P.compare_cells(a, c, where="chamber %d free run" % i, velocities=False,
                                            source=P.source_irradiance(orc.desc))
                 if not any(k in e for k in ("irradiance out", "t_local", "co2_local", "n2_local"))]
        assert b.chambers[i].counters()[3] == 0
    assert not errs, "\n".join(errs[:20])


# ---------------------------------------------------------------------------
# The analytic 3-D pins of the oracle (test_oracle_3d.py), run on the engine
# ---------------------------------------------------------------------------
import test_oracle_3d as O3  # noqa: E402


def engine(desc):
    return agb.World(desc)


@pytest.mark.parametrize("check", O3.CHECKS, ids=[c.__name__ for c in O3.CHECKS])
def test_engine_3d_analytic(check):
    check(engine)


@pytest.mark.parametrize("bcx", [(agb.BC_DIRICHLET, agb.BC_ROBIN), (agb.BC_ROBIN, agb.BC_DIRICHLET)])
def test_engine_stencil_faces(bcx):
    O3.check_stencil_reduces_to_1d(engine, bcx)


@pytest.mark.parametrize("direction", O3.DIRECTIONS)
def test_engine_column_shading(direction):
    O3.check_column_shading(engine, direction)
