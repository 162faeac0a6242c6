"""The scenario spine on the GPU: each of the reference's scenarios the engine
supports, and this suite's driven scenario, run through the spine on the
engine and on the oracle from the same scenario text. Integer cell state and
counts must stay equal tick for tick; fields, Stats and the measured accept
values within the floating-point tolerance."""
import glob
import json
import os

import numpy as np
import pytest

import helpers as H
import parity as P
import test_scenario as TS

agb = H.agb
S = H.load_scenario()
pytestmark = pytest.mark.gpu

SUPPORTED = ["first-light", "three-percent-line", "bloom", "komorov", "shadow-garden", "spin-drive-face",
             "taumoeba", "demo-herd", "sandbox"]
HAVE = {os.path.basename(p)[:-5] for p in glob.glob(os.path.join(TS.SCEN_DIR, "*.json"))}
MEASURE_RTOL = 1e-4        # correlations and fits over FP32-computed positions


def run_both(text, ticks):
    s = S.parse(text)
    gpu = S.instantiate(s)
    orc = S.instantiate(s, make_world=H.OracleWorld)
    for dw in (gpu, orc):
        for _ in range(ticks):
            S.apply_drive(dw)
            dw.step()
    return s, gpu, orc


def assert_tracks(s, gpu, orc, where):
    a, na = gpu.world.export_cells()
    b, nb = orc.world.export_cells()
    assert a.n == b.n and na == nb, where
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), "%s: %s" % (where, k)
    errs = P.compare_fields(gpu.world, orc.world, where=where)
    assert not errs, "\n".join(errs[:10])
    sg, so = gpu.world.stats(), orc.world.stats()
    for k in ("tick", "n_live", "n_dead", "n_awake", "n_dormant", "divisions_this_window", "deaths_this_window",
              "boil_events", "ignitions_this_window"):
        assert getattr(sg, k) == getattr(so, k), "%s: Stats.%s" % (where, k)
    for k in ("sim_time_s", "mean_charge", "total_energy_j", "mean_temp_medium_k", "max_temp_medium_k"):
        x, y = getattr(sg, k), getattr(so, k)
        assert abs(x - y) <= 1e-6 * abs(y) + 1e-9, "%s: Stats.%s %r vs %r" % (where, k, x, y)


@pytest.mark.parametrize("sid", SUPPORTED)
def test_reference_scenario_tracks_oracle(sid):
    if sid not in HAVE:
        pytest.skip("reference scenario files not present")
    s, gpu, orc = run_both(TS.text_of(sid), 30)
    assert_tracks(s, gpu, orc, sid)


def test_driven_scenario_tracks_oracle():
    s, gpu, orc = run_both(json.dumps(TS.DRIVEN), 45)
    assert gpu.world.count() == 1000
    assert_tracks(s, gpu, orc, "driven")


def test_measured_accept_values_agree():
    text = json.dumps(TS.DRIVEN)
    s = S.parse(text)
    res = []
    for make in (None, H.OracleWorld):
        dw = S.instantiate(s, make_world=make)
        ok, r = S.run_assert(s, dw, ticks=45, graph=make is None)
        res.append((ok, r))
    (ok_g, rg), (ok_o, ro) = res
    assert ok_g == ok_o
    for (m, vg, pg), (_m, vo, po) in zip(rg, ro):
        assert pg == po, m
        assert abs(vg - vo) <= MEASURE_RTOL * abs(vo) + 1e-6, (m, vg, vo)


def test_scenario_needing_a_missing_grid_refuses():
    if "taumoeba" not in HAVE:
        pytest.skip("reference scenario files not present")
    with pytest.raises(S.ScenarioUnsupported):
        S.instantiate(S.parse(TS.text_of("taumoeba")), grids={agb.FIELD_N2: agb.GridDesc()})


@pytest.mark.parametrize("sid", ["shadow-garden", "komorov", "bloom", "three-percent-line", "first-light",
                                 "spin-drive-face", "taumoeba"])
def test_reference_scenario_accepts(sid):
    """`--scenario ID --assert` at the scenario's own horizon (300 to 60,000
    ticks): the reference's acceptance gate, run on the engine, accepts."""
    if sid not in HAVE:
        pytest.skip("reference scenario files not present")
    s = S.parse(TS.text_of(sid))
    ok, res = S.run_assert(s, S.instantiate(s))
    assert ok, res
    assert len(res) == len(s.accept)


def test_headless_entry_point():
    """scenario.py's command line: ACCEPT exits 0, a file that does not parse 2."""
    import subprocess
    import sys
    import tempfile
    if "komorov" not in HAVE:
        pytest.skip("reference scenario files not present")
    script = os.path.join(H.PKG, "scenario.py")
    r = subprocess.run([sys.executable, script, "--scenario", "komorov", "--scenarios-dir", TS.SCEN_DIR, "--assert"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "scenario komorov: ACCEPT" in r.stdout
    with tempfile.NamedTemporaryFile("w", suffix=".json", delete=False) as fh:
        fh.write('{"objective": {"accept": [{"metric": "no_such_metric"}]}}')
    r = subprocess.run([sys.executable, script, "--scenario", fh.name, "--assert"],
                       capture_output=True, text=True, timeout=600)
    os.unlink(fh.name)
    assert r.returncode == 2 and "unknown accept metric" in r.stdout


@pytest.mark.parametrize("graph", [False, True])
def test_flash_tracks_oracle(graph):
    """The spin-drive flash armed for 12 ticks, then disarmed (taxis resumes):
    integer state equal to the oracle's, the audit within the FP tolerance."""
    import scenarios as TSD
    d = TSD.slab_desc(cap=900, light=(1.0, 0.0, 1e4, 0.0))
    d.taxis_enabled = 1
    sc = dict(desc=d, ticks=0,
              spawn=agb.spawn(800, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.004, awake=True))
    orc = H.OracleWorld(d)
    TSD.setup(orc, sc)
    gpu = agb.World(d)
    P.copy_state(orc, gpu)
    for k in range(18):
        on = k < 12
        gpu.set_flash(on)
        orc.set_flash(on)
        gpu.step(1, graph=graph)
        orc.step(1)
    a, _ = gpu.export_cells()
    b, _ = orc.export_cells()
    for k in P.INT_FIELDS:
        assert np.array_equal(a[k], b[k]), k
    gi, gd = gpu.flash_audit()
    oi, od = orc.flash_audit()
    assert od > 0.0
    assert abs(gd - od) <= 1e-9 * od and abs(gi - oi) <= 1e-9 * oi
    assert abs(gi * agb.C_LIGHT / gd - 1.0) < 1e-6
    assert gpu.counters()[3] == 0


def test_flash_armed_batch_chamber_equals_standalone():
    """A batch whose chamber has the flash armed leaves the staged path for the
    lanes path and still equals that chamber run on its own."""
    import test_gpu_batch as TB
    descs, spawns = TB.chambers()
    b = agb.Batch(descs, spawns, agb.batch_opts(lanes=2, staged=True))
    b.chambers[1].set_flash(True)
    for t in (2, 1):
        b.step(t)
    d, s = TB.chambers()
    w = TB.standalone(d[1], s[1], 0, walk=b.chambers[1].walk())
    w.set_flash(True)
    w.step(3)
    TB.assert_same(b.chambers[1], w, "flash chamber")
    for i in (0, 2, 3):
        d, s = TB.chambers()
        TB.assert_same(b.chambers[i], TB.standalone(d[i], s[i], 3, walk=b.chambers[i].walk()), "chamber %d" % i)


HEADLESS = os.path.join(H.PKG, "headless")
CHECKED = ["first-light", "three-percent-line", "bloom", "komorov", "shadow-garden", "spin-drive-face", "taumoeba"]


def _check_lines(text):
    return [ln.strip() for ln in text.splitlines() if ln.strip().startswith("[")]


@pytest.mark.parametrize("sid", CHECKED)
def test_native_runner_equals_python_spine(sid):
    """The native runner (headless.cpp over the C ABI) and the Python spine
    drive the engine through the same calls: the same measured values, printed
    the same way, over the first 300 ticks."""
    import io
    import subprocess
    if sid not in HAVE:
        pytest.skip("reference scenario files not present")
    s = S.parse(TS.text_of(sid))
    out = io.StringIO()
    S.run_assert(s, S.instantiate(s), ticks=300, out=out)
    r = subprocess.run([HEADLESS, "--scenario", sid, "--scenarios-dir", TS.SCEN_DIR, "--assert", "--ticks", "300"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode in (0, 1), r.stdout + r.stderr
    assert _check_lines(r.stdout) == _check_lines(out.getvalue())


def test_native_runner_accepts_and_is_deterministic():
    import subprocess
    if "komorov" in HAVE:
        r = subprocess.run([HEADLESS, "--scenario", "komorov", "--scenarios-dir", TS.SCEN_DIR, "--assert"],
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0 and "scenario komorov: ACCEPT" in r.stdout, r.stdout + r.stderr
    r = subprocess.run([HEADLESS, "--assert-deterministic", "--ticks", "200", "--cells", "3000"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "MATCH" in r.stdout, r.stdout + r.stderr
    r = subprocess.run([HEADLESS, "--scenario", "/no/such/file.json", "--assert"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 2
