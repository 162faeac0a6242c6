"""Pins the C oracle to the reference: every array after every stage of every
tick must carry the digest the reference's own sources produced
(tests/golden/*.json, made by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

import helpers as H
import scenarios as S

agb = H.agb
NAMES = sorted(S.scenarios().keys())


def load(name):
    with open(os.path.join(H.GOLDEN, name + ".json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_digests(name):
    sc = S.scenarios()[name]
    gold = load(name)
    w = H.OracleWorld(sc["desc"])
    rec, _ = S.trace(w, sc)
    assert rec["spawn"] == gold["spawn"], "spawn_kernel (src/sim/cell_store.cu:42-130)"
    assert rec["initial"] == gold["initial"]
    assert len(rec["steps"]) == len(gold["steps"])
    for got, want in zip(rec["steps"], gold["steps"]):
        where = "tick %d stage %s" % (want["tick"], want["stage"])
        for k in want["cells"]:
            assert got["cells"][k] == want["cells"][k], "%s: cell array %s" % (where, k)
        assert got["fields"] == want["fields"], where + ": fields"
        if "hash" in want:
            assert got["hash"] == want["hash"], where + ": hash"
        if "forces" in want:
            assert got["forces"] == want["forces"], where + ": forces"
    assert rec["snapshot_initial"] == gold["snapshot_initial"], "snapshot_to_bytes (src/sim/snapshot.cu:134-165)"
    assert rec["snapshot_final"] == gold["snapshot_final"], "snapshot after the last tick"
    assert rec["accum"] == gold["accum"], "fixed-point StatsAccum"
    assert rec["counters"] == gold["counters"]
    for k, v in gold["stats"].items():
        assert float(rec["stats"][k]) == v, "Stats." + k


def test_oracle_brushes_match_reference():
    """world_apply_brush (src/sim/step.cu:80-89): the fields after each stroke
    carry the digests the reference's own brush kernel produced."""
    gold = load("brushes")["brushes"]
    w = H.OracleWorld(S.brush_desc())
    assert S.brush_trace(w) == gold


def test_oracle_brush_rejects_bad_strokes():
    """Unknown kinds and non-finite strokes return InvalidArgument (status 3)."""
    w = H.OracleWorld(S.brush_desc())
    lib = H.oracle_lib()
    assert lib.orc_world_apply_brush(w.h, 9, 0.0, 0.0, 1e-4, 1.0) == 3
    assert lib.orc_world_apply_brush(w.h, agb.BRUSH_HEAT, float("nan"), 0.0, 1e-4, 1.0) == 3
    assert lib.orc_world_apply_brush(w.h, agb.BRUSH_HEAT, 0.0, 0.0, float("inf"), 1.0) == 3


def test_pcg32_reference_vectors():
    # pcg32_srandom_r(42, 54) then six draws: the PCG reference demo's published
    # output, which tests/physics/test_rng.cpp:16-22 also pins.
    out = np.zeros(6, np.uint32)
    H.oracle_lib().orc_pcg32_seed_draws(42, 54, 6, out.ctypes.data)
    assert [hex(int(x)) for x in out] == ["0xa15c02b7", "0x7b47f409", "0xba1d3330",
                                         "0x83d2f293", "0xbfa4784b", "0xcbed606e"]


def test_collinear_rear_cell_sees_exactly_zero():
    # T13 (tests/physics/test_emission.cu:73-133) through the reference's fixture.
    d = np.load(os.path.join(H.GOLDEN, "collinear_shadow_tick0.npz"))
    ir, e = d["cell_irradiance"], d["cell_energy"]
    assert ir[0] > 0.0 and e[0] > 0.0
    assert ir[1] == 0.0 and e[1] == 0.0


def test_golden_scenarios_exercise_lifecycle():
    g = load("lifecycle_compaction")
    assert g["steps"][-1]["cells"]["count"] > g["initial"]["count"], "divisions happened"
    assert g["counters"][1] > 0, "deaths happened"
    h = load("hot_field")
    assert h["stats"]["n_dead"] > 0 and h["stats"]["n_awake"] > 0


@pytest.mark.skipif(not H.ref_available(), reason="reference sources not present on this machine")
def test_oracle_matches_live_reference_longer_run():
    """Where the reference is built here, run 20 ticks of a fresh seed in both."""
    d = S.slab_desc(bio=1e6, compaction=1, seed=777)
    sp = agb.spawn(800, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.3, awake=True)
    r, o = H.RefWorld(d), H.OracleWorld(d)
    r.spawn(sp), o.spawn(sp)
    r.step(20), o.step(20)
    cr, _ = r.export_cells()
    co, _ = o.export_cells()
    for name, _ in agb.CELL_FIELDS:
        assert np.array_equal(cr[name], co[name]), name
    for f in range(4):
        assert np.array_equal(r.export_field(f), o.export_field(f))


def test_fnv1a64_engine_matches_restatement():
    """contracts/snapshot_v1.h fnv1a64: engine (host code, no GPU), oracle and a
    plain Python loop agree; the empty input leaves the offset basis."""
    lib = H.oracle_lib()
    rng = np.random.default_rng(3)
    for n in (0, 1, 7, 4096):
        data = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        h = 1469598103934665603
        for b in data:
            h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        buf = np.frombuffer(data, np.uint8)
        assert agb.fnv1a64(data) == h
        assert lib.orc_fnv1a64(buf.ctypes.data if n else None, n, 1469598103934665603) == h
