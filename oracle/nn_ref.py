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


# ---------------------------------------------------------------------------
# The whole surrogate network, forward and backward, rounding to BF16 at the
# same points as the engine (every stored activation and gradient tensor;
# the network output and the weight gradients stay FP32).
# ---------------------------------------------------------------------------
LAYERS = [(16, 32, 0, True), (32, 64, 1, True), (64, 128, 2, True), (128, 64, 2, True), (64, 32, 1, True),
          (32, 16, 0, False)]


def split_params(flat):
    """Flat FP32 parameters (each layer: [27, cout, cin] weights, then cout biases)."""
    out, k = [], 0
    for cin, cout, _lvl, _relu in LAYERS:
        n = 27 * cout * cin
        out.append((flat[k:k + n].reshape(27, cout, cin), flat[k + n:k + n + cout]))
        k += n + cout
    return out


def norm_constants(desc):
    """The input/output scaling the engine derives from its descriptor."""
    t_scale = desc["train_temperature_amplitude"] if desc["train_temperature_amplitude"] > 0 else 1.0
    c_scale = 0.3 * desc["init"][1] if desc["init"][1] > 0 else 1.0
    qt = desc["train_heat_per_step"] if desc["train_heat_per_step"] > 0 else 1.0
    qc = desc["train_uptake_per_step"] if desc["train_uptake_per_step"] > 0 else 1.0
    f32 = np.float32
    dt = f32(0.05 * f32(t_scale) + desc["steps"] * f32(qt))
    dc = f32(0.01 * f32(c_scale) + desc["steps"] * f32(qc))
    return dict(t_mean=f32(desc["init"][0]), t_scale=f32(t_scale), c_mean=f32(desc["init"][1]),
                c_scale=f32(c_scale), qt=f32(qt), qc=f32(qc), dt=dt, dc=dc,
                d1t=f32(dt / f32(desc["steps"])), d1c=f32(dc / f32(desc["steps"])))


def ftcs_step(x, coeff, bc, face, robin):
    """One 7-point FTCS pass in FP32, operation for operation as the engine's
    3-D kernel: c + coeff * (((((l + r) + d) + u) + b) + a - 6c), ghost values
    per face (Dirichlet: the face value; Robin: c - robin * (c - face);
    Neumann: c). x is [nz, ny, nx]; faces in x-, x+, y-, y+, z-, z+ order."""
    f32 = np.float32
    x = np.asarray(x, f32)
    robin = f32(robin)

    def ghost(k, c):
        if bc[k] == 0:
            return np.full_like(c, f32(face[k]))
        if bc[k] == 2:
            return (c - robin * (c - f32(face[k]))).astype(f32)
        return c

    def nb(axis, side, k):
        sl = [slice(None)] * 3
        out = np.empty_like(x)
        n = x.shape[axis]
        src = [slice(None)] * 3
        if side < 0:
            sl[axis] = slice(1, n); src[axis] = slice(0, n - 1)
            out[tuple(sl)] = x[tuple(src)]
            e = [slice(None)] * 3; e[axis] = slice(0, 1)
        else:
            sl[axis] = slice(0, n - 1); src[axis] = slice(1, n)
            out[tuple(sl)] = x[tuple(src)]
            e = [slice(None)] * 3; e[axis] = slice(n - 1, n)
        out[tuple(e)] = ghost(k, x[tuple(e)])
        return out

    l, r = nb(2, -1, 0), nb(2, 1, 1)
    d, u = nb(1, -1, 2), nb(1, 1, 3)
    b, a = nb(0, -1, 4), nb(0, 1, 5)
    s = ((((l + r) + d) + u) + b) + a
    s = (s - f32(6.0) * x).astype(f32)
    return (x + f32(coeff) * s).astype(f32)


def surrogate_grads(flat, T0, C0, qT, qC, T1, C1, nm, step_T, step_C):
    """Loss and flat gradients of one window; fields are [nz, ny, nx] float32.
    step_T / step_C apply one FTCS pass of each field (the network's d1 input)."""
    P = split_params(np.asarray(flat, np.float32))
    W = [bf16_round(w) for w, _ in P]
    B = [b.astype(np.float64) for _, b in P]
    f32 = np.float32
    x0 = np.zeros(T0.shape + (16,), np.float32)
    x0[..., 0] = (T0 - nm["t_mean"]) / nm["t_scale"]
    x0[..., 1] = (C0 - nm["c_mean"]) / nm["c_scale"]
    x0[..., 2] = qT / nm["qt"]
    x0[..., 3] = qC / nm["qc"]
    x0[..., 4] = (step_T((T0 + qT).astype(f32)) - T0) / nm["d1t"]
    x0[..., 5] = (step_C((C0 + qC).astype(f32)) - C0) / nm["d1c"]
    x0 = bf16_round(x0)
    r = lambda a: bf16_round(a.astype(np.float32))
    a1 = r(conv3(x0, W[0], B[0], relu=True))
    p1 = r(avgpool2(a1.astype(np.float64)))
    a2 = r(conv3(p1, W[1], B[1], relu=True))
    p2 = r(avgpool2(a2.astype(np.float64)))
    a3 = r(conv3(p2, W[2], B[2], relu=True))
    a4 = r(conv3(a3, W[3], B[3], relu=True))
    u2 = r(upsample2(a4).astype(np.float64) + a2)
    a5 = r(conv3(u2, W[4], B[4], relu=True))
    u1 = r(upsample2(a5).astype(np.float64) + a1)
    y = conv3(u1, W[5], B[5]).astype(np.float32)
    tgt = np.zeros_like(y)
    tgt[..., 0] = (T1 - T0) * (f32(1.0) / nm["dt"])
    tgt[..., 1] = (C1 - C0) * (f32(1.0) / nm["dc"])
    res = y - tgt
    loss = float((res[..., 0].astype(np.float64) ** 2 + res[..., 1].astype(np.float64) ** 2).mean())
    dy = r(res)
    g = [None] * 6
    g[5] = conv3_wgrad(u1, dy)
    du1 = r(conv3_dgrad(dy, W[5]))
    da5 = r(upsample2_backward(du1.astype(np.float64)) * (a5 > 0))
    g[4] = conv3_wgrad(u2, da5)
    du2 = r(conv3_dgrad(da5, W[4]))
    da4 = r(upsample2_backward(du2.astype(np.float64)) * (a4 > 0))
    g[3] = conv3_wgrad(a3, da4)
    da3 = r(conv3_dgrad(da4, W[3]) * (a3 > 0))
    g[2] = conv3_wgrad(p2, da3)
    dp2 = r(conv3_dgrad(da3, W[2]))
    da2 = r((0.125 * upsample2(dp2.astype(np.float64)) + du2) * (a2 > 0))
    g[1] = conv3_wgrad(p1, da2)
    dp1 = r(conv3_dgrad(da2, W[1]))
    da1 = r((0.125 * upsample2(dp1.astype(np.float64)) + du1) * (a1 > 0))
    g[0] = conv3_wgrad(x0, da1)
    flat_g = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in g])
    return loss, flat_g, y
