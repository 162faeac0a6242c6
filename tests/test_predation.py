"""Predation (src/sim/predation.cu) on the CPU: the oracle's restatement of the
predator store against the reference itself, where it is built here. A small
dense chamber, so that predators find prey every few ticks, digest on a fast
biology clock, divide with mutated tolerance and die in the nitrogen half of
the chamber; dead predators are compacted. Every array of both stores, bit
for bit, tick by tick."""
import numpy as np
import pytest

import helpers as H
import scenarios as S

agb = H.agb
needs_ref = pytest.mark.skipif(not H.ref_available(), reason="reference not built here")


def dense_predator_world():
    d = S.slab_desc(cap=4000, bio=2e5, compaction=1)
    d.chamber_w = d.chamber_h = 4.0e-4
    d.tau_capacity = 64
    d.tau_compaction_enabled = 1
    n2 = np.full((1, 32, 32), 0.0125, np.float32)
    n2[0, :, :16] = 0.0                     # lethal above tolerance 0.25 in the right half
    sp = agb.spawn(2500, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.3, awake=True)
    return d, sp, n2


def seed_world(world, d, sp, n2, tau=30, seed=77):
    world.spawn(sp)
    world.import_field(agb.FIELD_N2, n2)
    world.spawn_taumoeba(tau, seed)


def same_store(a, b, fields):
    return [name for name, _t in fields if a.n != b.n or not np.array_equal(a[name].view(np.uint8),
                                                                           b[name].view(np.uint8))]


@needs_ref
def test_predation_matches_reference():
    d, sp, n2 = dense_predator_world()
    r, o = H.RefWorld(d), H.OracleWorld(d)
    try:
        seed_world(r, d, sp, n2)
        seed_world(o, d, sp, n2)
        ta, _ = r.export_taumoeba()
        tb, _ = o.export_taumoeba()
        assert same_store(ta, tb, agb.TAU_FIELDS) == [], "taumoeba_spawn"
        saw = {"division": False, "engulf": False, "n2_death": False}
        for k in range(60):
            r.step(1)
            o.step(1)
            ta, na = r.export_taumoeba()
            tb, nb = o.export_taumoeba()
            assert na == nb and same_store(ta, tb, agb.TAU_FIELDS) == [], "tick %d: predators" % k
            ca, _ = r.export_cells()
            cb, _ = o.export_cells()
            assert same_store(ca, cb, agb.CELL_FIELDS) == [], "tick %d: cells" % k
            saw["division"] |= bool(np.any(tb["generation"] > 0))
            saw["engulf"] |= bool(np.any(tb["digest_timer"] > 0))
            saw["n2_death"] |= nb - 1 > tb.n
        assert all(saw.values()), saw
        so = o.stats()
        assert so.n_taumoeba == tb.n and so.mean_tau_tolerance > 0.0
    finally:
        r.close()


@needs_ref
def test_predator_snapshot_matches_reference():
    """snapshot_to_bytes with a predator store: the same bytes as the reference."""
    d, sp, n2 = dense_predator_world()
    r, o = H.RefWorld(d), H.OracleWorld(d)
    try:
        seed_world(r, d, sp, n2)
        seed_world(o, d, sp, n2)
        r.step(5)
        o.step(5)
        assert r.snapshot(b"tau") == o.snapshot(b"tau")
    finally:
        r.close()
