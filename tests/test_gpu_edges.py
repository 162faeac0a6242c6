"""Edge cases: an empty population, a single cell, a store that fills while
cells divide (divisions stop at capacity, the store never wraps), an import
larger than the store, and batches holding an empty or a full chamber. Each
runs from identical imported state against the oracle, or against standalone
worlds for the batch."""
import numpy as np
import pytest

import helpers as H
import parity as P
import scenarios as S
import test_gpu_batch as TB

agb = H.agb
pytestmark = pytest.mark.gpu
EMAX = agb.CELL_ENERGY_MAX


def seeded(sc):
    orc = H.OracleWorld(sc["desc"])
    S.setup(orc, sc)
    gpu = agb.World(sc["desc"])
    P.copy_state(orc, gpu)
    return gpu, orc


def run_both(sc, ticks, graph):
    gpu, orc = seeded(sc)
    for _ in range(ticks):
        gpu.step(1, graph=graph)
        orc.step(1)
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    return gpu, orc, a, b


@pytest.mark.parametrize("graph", [False, True])
def test_empty_world_ticks(graph):
    sc = dict(desc=S.slab_desc(cap=64), ticks=4, spawn=agb.spawn(0))
    gpu, orc, a, b = run_both(sc, 4, graph)
    assert a.n == b.n == 0
    assert P.compare_fields(gpu, orc, where="empty") == []
    st = gpu.stats()
    assert st.tick == 4 and st.n_live == 0 and st.n_dead == 0
    assert gpu.counters()[3] == 0


def test_single_cell_tracks_oracle():
    sc = dict(desc=S.slab_desc(cap=4), ticks=5,
              spawn=agb.spawn(1, charge_dist=agb.DIST_CONSTANT, charge_a=0.1, awake=True))
    gpu, orc = seeded(sc)
    gpu.step(1)
    orc.step(1)
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    errs = P.compare_cells(a, b, where="tick 0", scales=orc.export_term_scales(),
                           source=P.source_irradiance(sc["desc"]))
    assert not errs, "\n".join(errs)
    gpu.step(4, graph=True)
    orc.step(4)
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    assert a.n == b.n == 1
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), k


def _ready_to_divide(cells, desc):
    cells.a["energy"][:cells.n] = 0.9 * EMAX


@pytest.mark.parametrize("cells,cap", [(40, 64), (64, 64), (50, 60), (3, 100)])
def test_divisions_stop_at_capacity(cells, cap):
    """Every cell ready to divide, more than the free slots: the oracle's
    counts, ids, slots and RNG streams, whichever cells got a slot."""
    d = S.slab_desc(cap=cap)
    d.division_predicate = agb.DIVIDE_ENERGY
    d.division_energy = 0.5 * EMAX
    sc = dict(desc=d, ticks=3, mutate=_ready_to_divide, spawn=agb.spawn(cells, awake=True))
    gpu, orc, a, b = run_both(sc, 3, True)
    assert a.n == b.n <= cap
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), k
    sg, so = gpu.stats(), orc.stats()
    assert sg.divisions_this_window == so.divisions_this_window
    assert gpu.counters()[3] == 0


def test_import_beyond_capacity_is_rejected():
    w = agb.World(S.slab_desc(cap=16))
    with pytest.raises(agb.AgbError):
        w.import_cells(agb.CellArrays(17), 0)
    w.spawn(agb.spawn(8))
    w.step(1)
    assert w.count() == 8 and w.counters()[3] == 0


@pytest.mark.parametrize("staged", [True, False])
def test_batch_with_empty_and_full_chambers(staged):
    """A chamber with no cells and one whose store is full (its divisions are
    all refused) beside ordinary ones: each equals its standalone world."""
    descs, spawns = TB.chambers()
    spawns[1] = agb.spawn(0)
    descs[2].capacity = 1200                     # exactly its population: no free slot
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=staged))
    assert b.staged() == staged
    for t in (1, 2, 1):
        b.step(t)
    for i in range(b.n):
        d, s = TB.chambers()
        s[1] = agb.spawn(0)
        d[2].capacity = 1200
        w = TB.standalone(d[i], s[i], 4, walk=b.chambers[i].walk())
        TB.assert_same(b.chambers[i], w, "chamber %d" % i)
    assert b.chambers[1].count() == 0
    assert b.chambers[2].count() == 1200
