"""CPU restatement of the 3-D U-Net warm start (test infrastructure only).

The U-Net has no counterpart in the reference; this numpy version is the
checker for the library's tensor-core convolutions and for the gradients of
the whole network.  It rounds to BF16 at the same points as the device path
(activations, output gradients, data gradients, pooling and up-sampling
results) and sums convolutions in FP64, so differences against the device
come from the device's FP32 accumulation order alone.

Layout: tensors are [D, H, W, C] (channel fastest), convolution weights
[Cout, 27, Cin] with tap = 9 (dz + 1) + 3 (dy + 1) + (dx + 1), zero padding.
Parameters form one vector, layer by layer (weights, then biases), layers in
the order of ``layer_shapes``.
"""
from __future__ import annotations

import numpy as np

CH = (16, 32, 64, 128)
N_IN, N_OUT, PAD = 2, 4, 16


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), kept as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def layer_shapes():
    """(cin, cout, relu) of every convolution, in parameter order."""
    s = []
    for l in range(4):
        s.append((PAD if l == 0 else CH[l - 1], CH[l], True))
        s.append((CH[l], CH[l], True))
    for l in (2, 1, 0):
        low = CH[3] if l == 2 else CH[l + 1]
        s.append((low + CH[l], CH[l], True))
        s.append((CH[l], CH[l], True))
    s.append((CH[0], PAD, False))
    return s


def param_count():
    return sum(co * 27 * ci + co for ci, co, _ in layer_shapes())


def split_params(vec):
    out, o = [], 0
    for ci, co, _ in layer_shapes():
        w = vec[o:o + co * 27 * ci].reshape(co, 27, ci)
        o += co * 27 * ci
        b = vec[o:o + co]
        o += co
        out.append((w, b))
    return out


def _taps():
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def _shifted(x, dz, dy, dx):
    """x[z + dz, y + dy, x + dx] with zeros outside."""
    D, H, W, _ = x.shape
    p = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    return p[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]


def conv(x, w, b=None):
    """FP64 sum of the 3x3x3 convolution: y[v, co] = sum_tap,ci x[v + tap, ci] w[co, tap, ci] (+ b)."""
    x = x.astype(np.float64)
    w = w.astype(np.float64)
    y = np.zeros(x.shape[:3] + (w.shape[0],))
    for t, (dz, dy, dx) in enumerate(_taps()):
        y += _shifted(x, dz, dy, dx) @ w[:, t, :].T
    if b is not None:
        y += b
    return y


def conv_wgrad(x, gy):
    """gw[co, tap, ci] = sum_v gy[v, co] x[v + tap, ci]; gb[co] = sum_v gy[v, co]."""
    x = x.astype(np.float64)
    gy = gy.astype(np.float64)
    co, ci = gy.shape[-1], x.shape[-1]
    g2 = gy.reshape(-1, co)
    gw = np.zeros((co, 27, ci))
    for t, (dz, dy, dx) in enumerate(_taps()):
        gw[:, t, :] = g2.T @ _shifted(x, dz, dy, dx).reshape(-1, ci)
    return gw, g2.sum(0)


def conv_dgrad(gy, w):
    """gx[v, ci] = sum_tap,co gy[v - tap, co] w[co, tap, ci]."""
    gy = gy.astype(np.float64)
    w = w.astype(np.float64)
    gx = np.zeros(gy.shape[:3] + (w.shape[2],))
    for t, (dz, dy, dx) in enumerate(_taps()):
        gx += _shifted(gy, -dz, -dy, -dx) @ w[:, t, :]
    return gx


class _Mode:
    """BF16 rounding at the device's points in FP32 (default), or exact FP64."""

    def __init__(self, exact=False):
        self.dt = np.float64 if exact else np.float32
        self.rnd = (lambda a: np.asarray(a, np.float64)) if exact else bf16

    def c(self, v):
        return self.dt(v)


def pool(x, m=_Mode()):
    D, H, W, C = x.shape
    s = np.zeros((D // 2, H // 2, W // 2, C), m.dt)
    for k in range(8):
        s += x[(k >> 2)::2, ((k >> 1) & 1)::2, (k & 1)::2]
    return m.rnd(m.c(0.125) * s)


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_grad(g, m=_Mode()):
    D, H, W, C = g.shape
    s = np.zeros((D // 2, H // 2, W // 2, C), m.dt)
    for k in range(8):
        s += g[(k >> 2)::2, ((k >> 1) & 1)::2, (k & 1)::2]
    return m.rnd(s)


def forward(params, x_in, exact=False):
    """x_in [D, H, W, 2] -> (outputs [D, H, W, 4] before rounding, all 16
    output channels, saved activations).  exact: FP64 without rounding."""
    m = _Mode(exact)
    P = split_params(params)
    D, H, W, _ = x_in.shape
    x = np.zeros((D, H, W, PAD), m.dt)
    x[..., :N_IN] = x_in
    x = m.rnd(x)
    act = {"x": x}
    li = 0

    def layer(inp, relu=True):
        nonlocal li
        w, b = P[li]
        li += 1
        y = conv(inp, m.rnd(w)).astype(m.dt) + b.astype(m.dt)
        if relu:
            y = np.maximum(y, 0)
        return y

    inp = x
    for l in range(4):
        if l > 0:
            inp = act[f"p{l}"] = pool(act[f"e{l - 1}b"], m)
        act[f"e{l}a"] = m.rnd(layer(inp))
        act[f"e{l}b"] = m.rnd(layer(act[f"e{l}a"]))
    low = act["e3b"]
    for l in (2, 1, 0):
        act[f"c{l}"] = np.concatenate([up(low), act[f"e{l}b"]], axis=-1)
        act[f"d{l}a"] = m.rnd(layer(act[f"c{l}"]))
        act[f"d{l}b"] = m.rnd(layer(act[f"d{l}a"]))
        low = act[f"d{l}b"]
    out32 = layer(low, relu=False)
    act["out"] = m.rnd(out32)
    return out32[..., :N_OUT], out32, act


def loss_and_gradients(params, x_in, target, mask, exact=False):
    """Masked MSE over the 4 outputs and the gradient vector (parameter layout)."""
    m = _Mode(exact)
    P = split_params(params)
    _, out32, a = forward(params, x_in, exact)
    count = max(float(mask.sum()), 1.0) * N_OUT
    t = np.zeros_like(out32)
    t[..., :N_OUT] = target
    r = out32 - t
    mk = mask.astype(m.dt)[..., None]
    loss = float((mk * r * r).astype(np.float64).sum() / count)
    g_out = m.rnd(m.c(2.0) * mk * r * m.c(1.0 / count))
    grads = [None] * len(P)
    shapes = layer_shapes()

    def back(li, inp, out, gy, need_gx=True):
        w, _ = P[li]
        if shapes[li][2]:
            gy = np.where(out > 0, gy, 0).astype(m.dt)
        gw, gb = conv_wgrad(inp, gy)
        grads[li] = (gw, gb)
        return m.rnd(conv_dgrad(gy, m.rnd(w)).astype(m.dt)) if need_gx else None

    last = len(P) - 1
    g = back(last, a["d0b"], a["out"], g_out)
    li = last - 1
    gskip = {}
    for l in (0, 1, 2):
        g = back(li, a[f"d{l}a"], a[f"d{l}b"], g)
        li -= 1
        gc = back(li, a[f"c{l}"], a[f"d{l}a"], g)
        li -= 1
        lowc = gc.shape[-1] - a[f"e{l}b"].shape[-1]
        g = up_grad(gc[..., :lowc], m)       # gradient of the lower level's output
        gskip[l] = gc[..., lowc:]
    ge = g                                    # gradient of e3b
    for l in (3, 2, 1, 0):
        gea = back(2 * l + 1, a[f"e{l}a"], a[f"e{l}b"], ge)
        inp = a[f"p{l}"] if l > 0 else a["x"]
        gp = back(2 * l, inp, a[f"e{l}a"], gea, need_gx=l > 0)
        if l > 0:
            ge = m.rnd(gskip[l - 1] + m.c(0.125) * up(gp))
    vec = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return loss, vec.astype(m.dt)


def init_params(seed):
    """He-initialised parameters with the padding channels zero (a test
    network; the library initialises its own)."""
    rng = np.random.default_rng(seed)
    out = []
    shapes = layer_shapes()
    for i, (ci, co, relu) in enumerate(shapes):
        real_in = N_IN if i == 0 else ci
        real_out = co if relu else N_OUT
        w = np.zeros((co, 27, ci), np.float32)
        w[:real_out, :, :real_in] = rng.normal(0, np.sqrt(2.0 / (27 * real_in)), (real_out, 27, real_in))
        b = np.zeros(co, np.float32)
        b[:real_out] = rng.normal(0, 0.05, real_out)
        out += [w.ravel(), b]
    return np.concatenate(out).astype(np.float32)


def features(walls, periodic=(False, True, True), sdf_scale=0.125):
    """Network inputs of a wall array [nz, ny, nx] (non-zero = solid), the
    CPU restatement of mflbm_unet_features: solid mask and the signed exact
    Euclidean distance to the nearest voxel of the other kind (scipy's
    distance transform, positive in the fluid) times sdf_scale.  A periodic
    axis is padded by a full period on both sides, so that every minimum
    image lies inside the padded volume."""
    from scipy import ndimage
    solid = np.asarray(walls) != 0
    nz, ny, nx = solid.shape
    pw = [(n if p else 0,) * 2 for n, p in zip((nz, ny, nx), periodic[::-1])]
    s = np.pad(solid, pw, mode="wrap")
    d_f = ndimage.distance_transform_edt(~s)
    d_s = ndimage.distance_transform_edt(s)
    sl = tuple(slice(p[0], p[0] + n) for p, n in zip(pw, (nz, ny, nx)))
    x = np.empty((nz, ny, nx, 2), np.float32)
    x[..., 0] = solid
    x[..., 1] = (d_f - d_s)[sl] * sdf_scale
    return x
