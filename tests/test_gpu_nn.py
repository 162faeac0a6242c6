"""The surrogate's tensor-core layers against their CPU restatement
(oracle/nn_ref.py) on the same BF16 inputs: forward convolution (bias, ReLU,
mask, BF16 and FP32 outputs), input gradient through flipped weights, and the
weight/bias gradient. Tolerance: FP32 accumulation of exact BF16 products in a
different order, 1e-4 of the output scale; BF16 outputs 1/128 relative."""
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


def dev_bf16(a):
    return torch.from_numpy(R.to_bf16_bits(a).view(np.int16)).cuda()


def ptr(t):
    return None if t is None else t.data_ptr()


def rand(shape, seed, scale=1.0):
    return (np.random.default_rng(seed).standard_normal(shape) * scale).astype(np.float32)


CASES = [(4, 4, 32, 16, 32), (2, 4, 64, 32, 64), (4, 8, 32, 64, 128), (2, 2, 128, 128, 64),
         (2, 2, 64, 32, 16), (2, 4, 64, 64, 32), (2, 1, 128, 16, 16), (2, 2, 128, 256, 32),
         # the persistent row kernel (rows of 128 voxels, 16 or 32 input channels): a few tiles per
         # CTA; several tiles per CTA (stage and accumulator rings wrap); two tiles per row
         (3, 5, 128, 16, 32), (2, 3, 128, 32, 16), (3, 3, 128, 32, 32), (2, 3, 128, 16, 64),
         (16, 48, 128, 16, 32), (12, 40, 128, 32, 16), (3, 4, 256, 16, 32)]


@pytest.mark.parametrize("D,Hh,W,cin,cout", CASES)
def test_conv3_forward(D, Hh, W, cin, cout):
    lib = agb.load()
    x = R.bf16_round(rand((D, Hh, W, cin), 1))
    w = R.bf16_round(rand((27, cout, cin), 2, 1.0 / np.sqrt(27 * cin)))
    b = rand((cout,), 3, 0.1)
    want = R.conv3(x, w, b, relu=True)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.zeros(D * Hh * W * cout, dtype=torch.float32, device="cuda")
    xb, wb, bb = dev_bf16(x), dev_bf16(w), torch.from_numpy(b).cuda()
    rc = lib.agb_nn_conv3(ptr(xb), ptr(wb), ptr(bb), D, Hh, W, cin, cout, 1, None, ptr(out), 1, ptr(err), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got = out.cpu().numpy().reshape(want.shape)
    scale = np.abs(want).max() + 1e-30
    assert np.abs(got - want).max() <= 1e-4 * scale, np.abs(got - want).max() / scale
    # BF16 output of the same convolution, with a gradient mask.
    mask = R.bf16_round(rand((D, Hh, W, cout), 4))
    out16 = torch.zeros(D * Hh * W * cout, dtype=torch.int16, device="cuda")
    rc = lib.agb_nn_conv3(ptr(xb), ptr(wb), ptr(bb), D, Hh, W, cin, cout, 1, ptr(dev_bf16(mask)), ptr(out16), 0,
                          ptr(err), None)
    assert rc == 0
    g16 = R.from_bf16_bits(out16.cpu().numpy().view(np.uint16)).reshape(want.shape)
    w16 = np.where(mask > 0, want, 0.0)
    assert np.all(np.abs(g16 - w16) <= np.abs(w16) / 128 + 1e-4 * scale)


@pytest.mark.parametrize("D,Hh,W,cin,cout", [(4, 4, 32, 16, 32), (2, 4, 64, 32, 64), (2, 2, 128, 64, 128),
                                             (4, 8, 32, 128, 64), (2, 2, 128, 32, 16), (2, 4, 64, 64, 32)])
def test_conv3_wgrad_and_dgrad(D, Hh, W, cin, cout):
    lib = agb.load()
    x = R.bf16_round(rand((D, Hh, W, cin), 5))
    dy = R.bf16_round(rand((D, Hh, W, cout), 6))
    w = R.bf16_round(rand((27, cout, cin), 7, 0.05))
    dw_want, db_want = R.conv3_wgrad(x, dy)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nbytes = lib.agb_nn_wgrad_scratch_bytes(D, Hh, W, cin, cout)
    scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    dw = torch.zeros(27 * cout * cin, dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    xb, dyb = dev_bf16(x), dev_bf16(dy)
    rc = lib.agb_nn_wgrad(ptr(xb), ptr(dyb), D, Hh, W, cin, cout, ptr(dw), ptr(db), ptr(scratch), nbytes, ptr(err),
                          None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got = dw.cpu().numpy().reshape(dw_want.shape)
    scale = np.abs(dw_want).max()
    assert np.abs(got - dw_want).max() <= 1e-4 * scale, np.abs(got - dw_want).max() / scale
    assert np.abs(db.cpu().numpy() - db_want).max() <= 1e-4 * np.abs(db_want).max()
    # Input gradient: convolution of dy with the flipped weights.
    if R.flip(w).shape[1] in (16, 32, 64, 128):
        wf = torch.zeros(27 * cout * cin, dtype=torch.int16, device="cuda")
        assert lib.agb_nn_flip_weights(ptr(dev_bf16(w)), ptr(wf), cout, cin, None) == 0
        dx = torch.zeros(D * Hh * W * cin, dtype=torch.float32, device="cuda")
        assert lib.agb_nn_conv3(ptr(dyb), ptr(wf), None, D, Hh, W, cout, cin, 0, None, ptr(dx), 1, ptr(err),
                                None) == 0
        want = R.conv3_dgrad(dy, w)
        gdx = dx.cpu().numpy().reshape(want.shape)
        assert np.abs(gdx - want).max() <= 1e-4 * np.abs(want).max()
