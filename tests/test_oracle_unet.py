"""The CPU restatement of the U-Net (oracle/unet_oracle.py) checked on its
own: exact-mode gradients against central finite differences, the BF16
rounding against torch's, and the convolution against a direct loop."""
import numpy as np
import pytest

from oracle import unet_oracle as UO


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a = np.concatenate([rng.normal(size=20000).astype(np.float32) * 10.0 ** rng.integers(-30, 30, 20000),
                        np.array([0.0, -0.0, 1.0, 1.00390625, 1.01171875, 3.0e38, -1e-40], np.float32)])
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(UO.bf16(a).view(np.uint32), ref.view(np.uint32))


def test_convolution_and_its_gradients_match_direct_sums():
    rng = np.random.default_rng(4)
    D, H, W, ci, co = 3, 4, 5, 2, 3
    x = rng.normal(size=(D, H, W, ci))
    w = rng.normal(size=(co, 27, ci))
    gy = rng.normal(size=(D, H, W, co))
    y = UO.conv(x, w)
    ref = np.zeros_like(y)
    gw = np.zeros_like(w)
    gx = np.zeros_like(x)
    for z in range(D):
        for yy in range(H):
            for xx in range(W):
                for t in range(27):
                    dz, dy, dx = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
                    zz, y2, x2 = z + dz, yy + dy, xx + dx
                    if 0 <= zz < D and 0 <= y2 < H and 0 <= x2 < W:
                        ref[z, yy, xx] += w[:, t, :] @ x[zz, y2, x2]
                        gw[:, t, :] += np.outer(gy[z, yy, xx], x[zz, y2, x2])
                        gx[zz, y2, x2] += w[:, t, :].T @ gy[z, yy, xx]
    assert np.allclose(y, ref)
    gw2, gb2 = UO.conv_wgrad(x, gy)
    assert np.allclose(gw2, gw) and np.allclose(gb2, gy.reshape(-1, co).sum(0))
    assert np.allclose(UO.conv_dgrad(gy, w), gx)


def test_network_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = UO.init_params(1).astype(np.float64)
    D = 8
    x = rng.normal(size=(D, D, D, 2))
    t = rng.normal(size=(D, D, D, 4))
    m = (rng.random((D, D, D)) > 0.3).astype(np.float64)
    loss, g = UO.loss_and_gradients(p, x, t, m, exact=True)
    assert g.size == UO.param_count() == p.size

    def f(q):
        _, o, _ = UO.forward(q, x, exact=True)
        return float(((o[..., :4] - t) ** 2 * m[..., None]).sum() / (m.sum() * 4))

    assert abs(f(p) - loss) <= 1e-12 * abs(loss)
    idx = np.flatnonzero(np.abs(g) > 1e-6 * np.abs(g).max())
    # parameters of every layer: first, middle, deepest, decoder and final convolutions
    bounds = np.cumsum([0] + [co * 27 * ci + co for ci, co, _ in UO.layer_shapes()])
    sel = []
    for li in (0, 3, 7, 8, 12, 14):
        cand = idx[(idx >= bounds[li]) & (idx < bounds[li + 1])]
        sel += list(rng.choice(cand, 3, replace=False))
    for i in sel:
        h = 1e-5 * max(1.0, abs(p[i]))
        e = np.zeros_like(p)
        e[i] = h
        fd = (f(p + e) - f(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-4 * abs(g[i]) + 1e-10, (i, fd, g[i])
