"""The temperature flush is skipped while no cell has deposited heat.

Only awake, living cells exchange heat with the temperature grid
(src/sim/thermal.cu:19-71); while none does, every deposit word stays zero and
the reference's dense flush (src/fields/diffuse.cu:51-60) changes nothing, so
the engine's flush returns early. These worlds start with every cell dormant
under an ambient grid, so the first substeps flush nothing; a hot Dirichlet
x- face then heats the nearest layer past the ignition threshold and cells
there wake and start depositing. Across that transition, in a single world
and in a batched chamber beside one whose cells are awake from the start:
after every tick each temperature deposit word is zero (a flush skipped while
heat was pending would leave it there), and cells and fields stay within the
parity bounds of the oracle. (The exchange itself is FP32 per-cell physics,
so a deposit can differ from the oracle's FP64 one in its last fixed-point
unit: the fields are compared within the bounds, not bit for bit.)"""
import numpy as np
import pytest

import helpers as H
import parity as P

agb = H.agb
pytestmark = pytest.mark.gpu
TICKS = 12


def desc(seed, edge=32, face=600.0):
    d = agb.default_desc(capacity=4000, seed=seed, co2_init=1.0)
    d.chamber_w = d.chamber_h = d.chamber_d = 1.0e-3
    d.grid[agb.FIELD_T] = agb.grid(edge, edge, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9,
                                   [agb.BC_DIRICHLET] + [agb.BC_ROBIN] * 5,
                                   face_value=[face] + [agb.AMBIENT_TEMP_DEFAULT] * 5)
    d.grid[agb.FIELD_CO2] = agb.grid(edge, edge, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.GridDesc()
    d.grid[agb.FIELD_IRR] = agb.grid(edge, edge, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
    d.taxis_enabled = 0
    d.light = agb.Light(0.0, 0.0, 1.0, 1.0e4, 0.0, 1)
    return d


def awake_count(w):
    cells, _ = w.export_cells()
    f = cells["flags"]
    return int(np.count_nonzero(((f & agb.FLAG_OCCUPIED) != 0) & ((f & agb.FLAG_AWAKE) != 0)))


def flush_errors(gpu, orc, where):
    """Every temperature deposit folded in, and the fields within the bounds."""
    errs = P.compare_fields(gpu, orc, where=where)
    left = int(np.count_nonzero(gpu.export_deposit(agb.FIELD_T)))
    if left:
        errs.append("%s: %d temperature deposit words left unflushed" % (where, left))
    return errs


def test_single_world_wakes_and_flushes():
    d = desc(21)
    orc = H.OracleWorld(d)
    orc.spawn(agb.spawn(2000, charge_dist=agb.DIST_UNIFORM, charge_a=0.05, charge_b=0.2, awake=False))
    gpu = agb.World(d)
    P.copy_state(orc, gpu)
    assert awake_count(gpu) == 0
    errs, awake = [], []
    for t in range(TICKS):
        gpu.step(1, graph=True)
        orc.step(1)
        errs += flush_errors(gpu, orc, "tick %d" % t)
        a, _ = gpu.export_cells()
        b, _ = orc.export_cells()
        errs += P.compare_cells(a, b, where="tick %d" % t, scales=orc.export_term_scales(),
                                source=P.source_irradiance(d))
        awake.append(awake_count(gpu))
        P.copy_state(orc, gpu)
    assert gpu.counters()[3] == 0
    assert not errs, "\n".join(errs[:20])
    # The run crosses the transition it is about: cells woke after dormant substeps.
    assert awake[-1] > 0, awake


def test_batched_chamber_wakes_and_flushes():
    descs = [desc(31), desc(32, edge=40)]
    spawns = [agb.spawn(1500, charge_dist=agb.DIST_UNIFORM, charge_a=0.05, charge_b=0.2, awake=False),
              agb.spawn(1500, charge_dist=agb.DIST_UNIFORM, charge_a=0.05, charge_b=0.2, awake=True)]
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=1, staged=True))
    orcs = []
    for i in range(b.n):
        dd = agb.WorldDesc.from_buffer_copy(b.descs[i])
        dd.hash_cell_size = b.tuning(i).hash_cell_size
        orc = H.OracleWorld(dd)
        P.copy_state(b.chambers[i], orc)
        orcs.append(orc)
    assert awake_count(b.chambers[0]) == 0
    errs = []
    for t in range(TICKS):
        b.step(1)
        for i, orc in enumerate(orcs):
            orc.step(1)
            errs += flush_errors(b.chambers[i], orc, "chamber %d tick %d" % (i, t))
            P.copy_state(orc, b.chambers[i])
    for i in range(b.n):
        assert b.chambers[i].counters()[3] == 0
    assert not errs, "\n".join(errs[:20])
    assert awake_count(b.chambers[0]) > 0
