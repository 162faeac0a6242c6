"""Graph pre-capture (agb_world_prepare_graphs) and the in-graph section timers
(agb_world_set_timing / agb_world_section_times): neither changes results."""
import numpy as np
import pytest

import helpers as H
import parity as P
from test_gpu_parity3d import batch_chambers

agb = H.agb
pytestmark = pytest.mark.gpu


def world_pair():
    descs, spawns = batch_chambers()
    d, sp = descs[3], spawns[3]                 # 6,000 cells, 64^3 grids, compaction every third tick
    a = agb.World(d)
    a.spawn(sp)
    b = agb.World(d)
    P.copy_state(a, b)
    return a, b


def same(a, b):
    x, nx = a.export_cells()
    y, ny = b.export_cells()
    assert nx == ny and x.n == y.n
    for name, _t in agb.CELL_FIELDS:
        assert np.array_equal(x[name].view(np.uint8), y[name].view(np.uint8)), name
    for f in range(4):
        if a.desc.grid[f].nx > 0:
            assert np.array_equal(a.export_field(f).view(np.uint32), b.export_field(f).view(np.uint32)), f


def test_prepare_graphs_leaves_state_and_results_unchanged():
    a, b = world_pair()
    a.prepare_graphs(1)
    same(a, b)                                   # nothing ran
    k0 = a.graph_kernels()
    for _ in range(7):
        a.step(1, graph=True)
    b.step(7)
    same(a, b)
    assert a.graph_kernels() > k0
    assert a.counters()[3] == 0


def test_section_timers_time_the_graph_and_change_nothing():
    a, b = world_pair()
    a.set_timing(True)
    for _ in range(4):
        a.step(1, graph=True)
    t = a.section_times()
    b.step(4)
    same(a, b)
    for k in a.SECTIONS:
        assert k in t and t[k] > 0.0, (k, t)
        assert t[k] <= t["tick"] * 1.0001 + 1e-3, (k, t)
    a.set_timing(False)
    assert a.section_times() == {}
