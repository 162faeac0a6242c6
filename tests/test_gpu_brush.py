"""world_apply_brush (src/sim/step.cu:80-89) on the GPU: the reference's
strokes bit for bit on its slab grids, the same disc on every plane of 3-D
grids against the oracle, strokes between graph-replayed ticks, and the
error behaviour."""
import json
import os

import numpy as np
import pytest

import helpers as H
import parity as P
import scenarios as S
import test_gpu_batch as TB

agb = H.agb
pytestmark = pytest.mark.gpu


def test_brushes_match_reference_digests():
    with open(os.path.join(H.GOLDEN, "brushes.json")) as fh:
        gold = json.load(fh)["brushes"]
    w = agb.World(S.brush_desc())
    assert S.brush_trace(w) == gold


def test_brush_on_3d_grids_equals_oracle():
    d = TB.cube_desc(40, 64, seed=5)
    e = d.grid[agb.FIELD_T].nx
    d.grid[agb.FIELD_N2] = agb.grid(e, e, agb.N2_DIFFUSIVITY, 0.2, 1e15, agb.BC_NEUMANN)
    gpu, orc = agb.World(d), H.OracleWorld(d)
    half = 0.5 * d.chamber_w
    strokes = [(agb.BRUSH_HEAT, 0.1 * half, -0.2 * half, 0.4 * half, 3.0),
               (agb.BRUSH_CHILL, half, half, 0.5 * half, 1.5),
               (agb.BRUSH_INJECT_CO2, 0.0, 0.0, 10.0 * d.chamber_w, 0.25),
               (agb.BRUSH_INJECT_N2, -0.6 * half, 0.3 * half, 0.05 * half, 2.0)]
    for kind, x, y, r, s in strokes:
        gpu.apply_brush(kind, x, y, r, s)
        orc.apply_brush(kind, x, y, r, s)
        for f in (agb.FIELD_T, agb.FIELD_CO2, agb.FIELD_N2):
            a, b = gpu.export_field(f), orc.export_field(f)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (kind, f)
    t = gpu.export_field(agb.FIELD_T)
    assert np.array_equal(t[0], t[-1]), "the disc is the same on every plane"


@pytest.mark.parametrize("graph", [False, True])
def test_strokes_between_ticks_track_oracle(graph):
    """Heat and CO2 strokes land between ticks (as the reference's scenario
    driver issues them); replayed graphs see the new field values."""
    sc = dict(desc=S.slab_desc(cap=600), ticks=6,
              spawn=agb.spawn(500, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.3, awake=True))
    orc = H.OracleWorld(sc["desc"])
    S.setup(orc, sc)
    gpu = agb.World(sc["desc"])
    P.copy_state(orc, gpu)
    for t in range(6):
        stroke = (agb.BRUSH_HEAT if t % 2 == 0 else agb.BRUSH_INJECT_CO2, 2e-4 * t, -1e-4 * t, 6e-4, 0.5 + t)
        gpu.apply_brush(*stroke)
        orc.apply_brush(*stroke)
        gpu.step(1, graph=graph)
        orc.step(1)
    assert P.compare_fields(gpu, orc, where="brushed") == []
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), k


def test_brush_errors():
    d = S.brush_desc()
    d.grid[agb.FIELD_N2] = agb.GridDesc()
    w = agb.World(d)
    before = w.export_field(agb.FIELD_T)
    with pytest.raises(agb.AgbError):
        w.apply_brush(7, 0.0, 0.0, 1e-4, 1.0)
    with pytest.raises(agb.AgbError):
        w.apply_brush(agb.BRUSH_HEAT, float("nan"), 0.0, 1e-4, 1.0)
    with pytest.raises(agb.AgbError):
        w.apply_brush(agb.BRUSH_INJECT_N2, 0.0, 0.0, 1e-4, 1.0)
    w.apply_brush(agb.BRUSH_HEAT, 0.0, 0.0, 0.0, 5.0)
    w.apply_brush(agb.BRUSH_HEAT, 0.0, 0.0, -1.0, 5.0)
    assert np.array_equal(w.export_field(agb.FIELD_T), before)
    w.step(1)
    assert w.counters()[3] == 0
