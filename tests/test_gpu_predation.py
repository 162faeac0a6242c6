"""Predation on the GPU against the oracle: the seeded predator spawn, then
ticks from identical state (cells, fields and predators copied from the
oracle) in the dense chamber where predators engulf, digest, divide, die in
nitrogen and are compacted. Integer state exact; positions, velocities and
biomass within the floating-point tolerance (the predators' Gaussian draws
use CUDA's FP64 log/sin/cos, the oracle the host's, equal to the last ulp or
two). Also: graph replay equals eager stepping, Stats, the snapshot bytes, and
a batch holding a predator world."""
import numpy as np
import pytest

import helpers as H
import parity as P
import test_predation as TP

agb = H.agb
pytestmark = pytest.mark.gpu
TAU_INT = ("id", "flags", "generation", "target", "rng_state")
TAU_FP = ("x", "y", "z", "vx", "vy", "vz", "dir_x", "dir_y", "dir_z", "biomass", "prey_biomass",
          "digest_timer", "tolerance", "density_ema", "run_timer")


def seeded_pair():
    d, sp, n2 = TP.dense_predator_world()
    orc = H.OracleWorld(d)
    TP.seed_world(orc, d, sp, n2)
    gpu = agb.World(d)
    P.copy_state(orc, gpu)
    tau, nid = orc.export_taumoeba()
    gpu.import_taumoeba(tau, nid)
    return gpu, orc


def compare_tau(a, b, where, rtol=1e-9):
    assert a.n == b.n, where
    for k in TAU_INT:
        assert np.array_equal(a[k], b[k]), "%s: %s" % (where, k)
    for k in TAU_FP:
        x, y = a[k].astype(np.float64), b[k].astype(np.float64)
        assert np.all(np.abs(x - y) <= rtol * np.abs(y) + 1e-6 * np.abs(y).max() + 1e-300), "%s: %s" % (where, k)


def test_spawn_matches_oracle():
    d, sp, n2 = TP.dense_predator_world()
    gpu, orc = agb.World(d), H.OracleWorld(d)
    gpu.spawn_taumoeba(40, 123)
    orc.spawn_taumoeba(40, 123)
    a, na = gpu.export_taumoeba()
    b, nb = orc.export_taumoeba()
    assert na == nb == 41
    for k in ("x", "y", "z") + TAU_INT:
        assert np.array_equal(a[k], b[k]), k                  # uniform placement is exact arithmetic
    for k in ("dir_x", "dir_y", "dir_z"):
        assert np.all(np.abs(a[k] - b[k]) <= 2.5e-7), k       # one float ulp at most
    with pytest.raises(agb.AgbError):
        gpu.spawn_taumoeba(30, 1)                             # 41 + 30 > 64


@pytest.mark.parametrize("graph", [False, True])
def test_predation_tracks_oracle(graph):
    gpu, orc = seeded_pair()
    for k in range(20):
        gpu.step(1, graph=graph)
        orc.step(1)
    ta, na = gpu.export_taumoeba()
    tb, nb = orc.export_taumoeba()
    assert na == nb
    compare_tau(ta, tb, "after 20 ticks")
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    assert a.n == b.n
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), k
    assert int(np.sum(tb["generation"] > 0)) > 0 and int(np.sum(tb["digest_timer"] > 0)) > 0
    sg, so = gpu.stats(), orc.stats()
    assert sg.n_taumoeba == so.n_taumoeba and sg.n_live == so.n_live and sg.n_dead == so.n_dead
    assert abs(sg.mean_tau_tolerance - so.mean_tau_tolerance) <= 1e-6
    assert gpu.counters()[3] == 0


def test_graph_equals_eager_with_predators():
    g1, _ = seeded_pair()
    g2, _ = seeded_pair()
    g1.step(9)
    for _ in range(3):
        g2.step(3, graph=True)
    a, _ = g1.export_taumoeba()
    b, _ = g2.export_taumoeba()
    for k, _t in agb.TAU_FIELDS:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_snapshot_with_predators_equals_oracle():
    gpu, orc = seeded_pair()
    data = gpu.snapshot(b"tau")
    assert data == orc.snapshot(b"tau")
    w2 = agb.snapshot_load(gpu.desc, data)
    a, _ = w2.export_taumoeba()
    b, _ = gpu.export_taumoeba()
    for k, _t in agb.TAU_FIELDS:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_batch_chamber_with_predators_equals_standalone():
    import test_gpu_batch as TB
    descs, spawns = TB.chambers()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=True))
    b.chambers[2].spawn_taumoeba(12, 9)
    for t in (2, 1):
        b.step(t)
    d, s = TB.chambers()
    w = TB.standalone(d[2], s[2], 0, walk=b.chambers[2].walk())
    w.spawn_taumoeba(12, 9)
    w.step(3)
    TB.assert_same(b.chambers[2], w, "predator chamber")
    x, _ = b.chambers[2].export_taumoeba()
    y, _ = w.export_taumoeba()
    for k, _t in agb.TAU_FIELDS:
        assert np.array_equal(x[k].view(np.uint8), y[k].view(np.uint8)), k
