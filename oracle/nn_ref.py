"""CPU restatement of the field surrogate's layers (test infrastructure only).

The surrogate has no counterpart in the reference, so this file is the
oracle for it: the same layer definitions as the engine's tensor-core and
memory-bound kernels, in float64 numpy, on BF16-rounded inputs. Layouts match
the engine: activations channels-last [D, H, W, C]; weights [27, Cout, Cin],
tap t = (dz+1)*9 + (dy+1)*3 + (dx+1); 3x3x3 "same" convolutions with zero
padding."""
import numpy as np


def bf16_round(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def to_bf16_bits(a):
    """float32 -> uint16 bit patterns of the bfloat16 rounding."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def taps():
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                yield (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1), dz, dy, dx


def shifted(x, dz, dy, dx):
    """x[z+dz, y+dy, x+dx, :] with zeros outside the grid."""
    D, H, W, C = x.shape
    p = np.zeros((D + 2, H + 2, W + 2, C), x.dtype)
    p[1:-1, 1:-1, 1:-1] = x
    return p[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]


def conv3(x, w, bias=None, relu=False):
    """out[m, co] = sum_t sum_ci w[t, co, ci] * x_t[m, ci] (+ bias, ReLU)."""
    x = x.astype(np.float64)
    w = w.astype(np.float64)
    D, H, W, C = x.shape
    out = np.zeros((D, H, W, w.shape[1]))
    for t, dz, dy, dx in taps():
        out += shifted(x, dz, dy, dx) @ w[t].T
    if bias is not None:
        out += bias
    if relu:
        out = np.maximum(out, 0.0)
    return out


def conv3_wgrad(x, dy):
    """dw[t, co, ci] = sum_m dy[m, co] * x_t[m, ci]; db[co] = sum_m dy[m, co]."""
    x = x.astype(np.float64)
    dy = dy.astype(np.float64)
    C = x.shape[-1]
    Co = dy.shape[-1]
    dw = np.zeros((27, Co, C))
    d2 = dy.reshape(-1, Co)
    for t, dz, dyy, dx in taps():
        dw[t] = d2.T @ shifted(x, dz, dyy, dx).reshape(-1, C)
    return dw, d2.sum(0)


def conv3_dgrad(dy, w):
    """Gradient with respect to the input: the convolution with flipped, transposed weights."""
    return conv3(dy, flip(w))


def flip(w):
    """wf[26 - t, ci, co] = w[t, co, ci]."""
    return np.ascontiguousarray(w[::-1].transpose(0, 2, 1))


def avgpool2(x):
    D, H, W, C = x.shape
    return x.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(1, 3, 5))


def upsample2(x):
    return x.repeat(2, 0).repeat(2, 1).repeat(2, 2)


def upsample2_backward(dy):
    D, H, W, C = dy.shape
    return dy.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(1, 3, 5))
