"""The learned field surrogate: gradients of the engine's own forward and
backward kernels against the CPU restatement (oracle/nn_ref.py), training on
seeded FTCS windows, and the judge that falls back to the plain stencil.

Gradient tolerance: both sides round every stored tensor to BF16 at the same
points; FP32 (GPU) against FP64 (CPU) accumulation can flip a rounding now and
then, so each layer's weight gradient must agree to 2 % in relative L2 norm
and 0.999 in cosine."""
import importlib.util
import os

import numpy as np
import pytest

import helpers as H

agb = H.agb
torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_spec = importlib.util.spec_from_file_location("nn_ref", os.path.join(H.ROOT, "oracle", "nn_ref.py"))
R = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(R)


def fields(shape, n=4):
    return [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(n)]


def small_desc(**kw):
    d = agb.surrogate_desc(nx=128, ny=16, nz=8, extent=4.0e-3)
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_gradients_match_cpu_oracle():
    d = small_desc(seed=3)
    sg = agb.Surrogate(d)
    shape = (d.nz, d.ny, d.nx)
    T, Cf, qT, qC = fields(shape)
    sg.window(7, T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr())
    T1, C1 = T.clone(), Cf.clone()
    sg.reference(T1.data_ptr(), C1.data_ptr(), qT.data_ptr(), qC.data_ptr())
    # Non-trivial weights everywhere (the last layer starts near zero).
    rng = np.random.default_rng(0)
    p = sg.params()
    p = (p + 0.02 * rng.standard_normal(p.size)).astype(np.float32)
    sg.set_params(p)
    loss, g = sg.gradients(T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr(), T1.data_ptr(), C1.data_ptr())
    assert sg.error_word() == 0
    host = [x.cpu().numpy() for x in (T, Cf, qT, qC, T1, C1)]
    dd = d.as_dict()
    nm = R.norm_constants(dd)
    dx = dd["extent"] / dd["nx"]
    robin = np.float32(dx * agb.AIR_CONVECTION_H / agb.WATER_CONDUCTIVITY)
    coeff = [np.float32(dd["diffusivity"][f] * dd["dt"] / (dx * dx)) for f in range(2)]
    step_T = lambda x: R.ftcs_step(x, coeff[0], dd["bc"][0], dd["face"][0], robin)
    step_C = lambda x: R.ftcs_step(x, coeff[1], dd["bc"][1], dd["face"][1], robin)
    want_loss, want_g, _y = R.surrogate_grads(p, *host, nm, step_T, step_C)
    assert abs(loss - want_loss) <= 1e-3 * want_loss
    k = 0
    for i, (cin, cout, _l, _r) in enumerate(R.LAYERS):
        n = 27 * cout * cin + cout
        a, b = g[k:k + n].astype(np.float64), want_g[k:k + n]
        k += n
        rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
        assert rel < 2e-2 and cos > 0.999, "layer %d: rel %.3g cos %.6f" % (i, rel, cos)


SD = H.load_surrogate_data()
W = H.load_workloads()


def test_training_on_world_windows_beats_untrained_and_persistence():
    """What the trained network gains, at the benchmark's setting: trained on
    windows cut from runs of the plain-step workloads (fields plus the cells'
    rasterised heat and uptake sources), on held-out windows from other runs
    its RMS error against the FTCS window is below persistence's (leaving the
    fields as they are, the method's baseline without a model) and less than
    half the untrained network's. Its largest error is not: at a few voxels
    holding strong cell heat sources it exceeds persistence's many times over
    (the benchmark reports both), so the judge's fallback stays in charge."""
    desc, _sp, _info = W.workload("slab25k", seed=1)
    sd = SD.surrogate_desc_for(desc, seed=5)
    sg = agb.Surrogate(sd)
    held = list(SD.world_windows(sd, 6, seed=900, every=7))
    before = SD.evaluate(sg, held)
    losses = [sg.train_on(*[x.data_ptr() for x in win]) for win in SD.world_windows(sd, TRAIN_WINDOWS, seed=100)]
    assert sg.error_word() == 0 and np.all(np.isfinite(losses))
    after = SD.evaluate(sg, held)
    print("untrained", before, "trained", after)
    assert after["net_rms_K"] < WORLD_RMS_GAIN * after["persistence_rms_K"]
    assert after["net_rms_K"] < 0.5 * before["net_rms_K"]


TRAIN_WINDOWS = 400
RMS_GAIN = 0.5            # synthetic windows: measured 0.30 (0.112 K against 0.377 K)
WORLD_RMS_GAIN = 0.85     # world windows: measured 0.69 (3.37 K against 4.88 K)


def test_training_beats_untrained_and_persistence():
    """What the trained network gains on the seeded synthetic windows at the
    benchmark's normalisation (20 K temperature excursions, 2 K/step heat
    sources): on held-out windows its RMS error against the FTCS window is
    far below the untrained network's and below persistence's."""
    desc, _sp, _info = W.workload("slab25k", seed=1)
    d = SD.surrogate_desc_for(desc, seed=5)         # 128^3, 16 steps
    sg = agb.Surrogate(d)
    shape = (d.nz, d.ny, d.nx)
    held = []
    for idx in (10 ** 6, 10 ** 6 + 1, 10 ** 6 + 2):
        f = fields(shape)
        sg.window(idx, *[x.data_ptr() for x in f])
        held.append(f)
    before = SD.evaluate(sg, held)
    losses = sg.train(TRAIN_WINDOWS)
    assert sg.error_word() == 0
    assert np.all(np.isfinite(losses))
    assert losses[-50:].mean() < 0.2 * losses[:20].mean()
    after = SD.evaluate(sg, held)
    print("untrained", before, "trained", after)
    assert after["net_rms_K"] < 0.5 * before["net_rms_K"]
    assert after["net_rms_K"] < RMS_GAIN * after["persistence_rms_K"]


def test_judge_falls_back_to_ftcs():
    d = agb.surrogate_desc(seed=9, judge_every=2)
    sg = agb.Surrogate(d)
    shape = (d.nz, d.ny, d.nx)
    T, Cf, qT, qC = fields(shape)
    sg.window(3, T.data_ptr(), Cf.data_ptr(), qT.data_ptr(), qC.data_ptr())
    ref_T, ref_C = T.clone(), Cf.clone()
    sg.reference(ref_T.data_ptr(), ref_C.data_ptr(), qT.data_ptr(), qC.data_ptr())
    # Call 1: not judged (judge_every = 2): the untrained network's output.
    r1 = sg.advance(T.clone().data_ptr(), Cf.clone().data_ptr(), qT.data_ptr(), qC.data_ptr())
    assert r1.judged == 0 and r1.last_used_surrogate == 1
    # Call 2: judged; the untrained network misses by far more than 0.01 K,
    # so the output is exactly the plain FTCS window.
    T2, C2 = T.clone(), Cf.clone()
    r2 = sg.advance(T2.data_ptr(), C2.data_ptr(), qT.data_ptr(), qC.data_ptr())
    assert r2.judged == 1 and r2.fallbacks == 1 and r2.last_used_surrogate == 0
    assert r2.last_err_temperature > 0.01
    assert torch.equal(T2, ref_T) and torch.equal(C2, ref_C)
    # A forced judge with loose tolerances keeps the network's output.
    d2 = agb.surrogate_desc(seed=9, tol_temperature=1e9, tol_energy=1e9)
    sg2 = agb.Surrogate(d2)
    T3 = T.clone()
    r3 = sg2.advance(T3.data_ptr(), Cf.clone().data_ptr(), qT.data_ptr(), qC.data_ptr(), judge=1)
    assert r3.judged == 1 and r3.fallbacks == 0 and r3.last_used_surrogate == 1
    assert not torch.equal(T3, ref_T)


def world_with_surrogate(tol, judge_every, cells=2000):
    d = agb.default_desc(capacity=2 * cells, seed=4, co2_init=1.0)
    d.chamber_w = d.chamber_h = d.chamber_d = 4.0e-3
    d.grid[agb.FIELD_T] = agb.grid(128, 128, agb.WATER_THERMAL_DIFFUSIVITY, agb.AMBIENT_TEMP_DEFAULT, 1e9,
                                   agb.BC_ROBIN)
    d.grid[agb.FIELD_CO2] = agb.grid(128, 128, agb.CO2_DIFFUSIVITY_WATER, 1.0, 1e15, agb.BC_NEUMANN)
    d.grid[agb.FIELD_N2] = agb.GridDesc()
    d.grid[agb.FIELD_IRR] = agb.grid(128, 128, agb.IRRADIANCE_NOMINAL_DIFFUSIVITY, 0.0, 1e18, agb.BC_NEUMANN)
    d.taxis_enabled = 0
    d.light = agb.Light(1.0, 0.0, 0.0, 1.0e4, 0.0, 1)
    w = agb.World(d)
    w.spawn(agb.spawn(cells, charge_dist=agb.DIST_UNIFORM, charge_a=0.0, charge_b=0.2, awake=True))
    sd = agb.surrogate_desc(seed=2, judge_every=judge_every, tol_temperature=tol, tol_energy=1e9 if tol > 1 else tol)
    sg = agb.Surrogate(sd)
    w.attach_surrogate(sg)
    return w, sg


def test_world_driven_by_surrogate():
    # Loose tolerance: every window is the network's; the world keeps stepping.
    w, sg = world_with_surrogate(1e9, 2)
    n0 = w.count()
    w.step(32)                                      # two windows, one judged
    r = sg.report()
    assert r.calls == 2 and r.judged == 1 and r.fallbacks == 0
    t = w.export_field(agb.FIELD_T)
    assert np.all(np.isfinite(t)) and w.count() == n0 and sg.error_word() == 0
    w.attach_surrogate(None)                        # back to per-tick FTCS
    w.step(2)
    assert np.all(np.isfinite(w.export_field(agb.FIELD_T)))
    # Zero tolerance: every judged window falls back to the plain FTCS window.
    w2, sg2 = world_with_surrogate(0.0, 1)
    w2.step(48)
    r2 = sg2.report()
    assert r2.calls == 3 and r2.judged == 3 and r2.fallbacks == 3 and r2.last_used_surrogate == 0
