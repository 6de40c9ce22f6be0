"""The separable exact distance transform of the warm-start inputs
(mf-lbm-cuda_gb300/csrc/unet_kernels.cuh: edt_axis_kernel and
edt_features_kernel), restated in numpy: three passes, x then y then z, each
taking at every voxel the minimum over its line of (squared distance so far +
offset^2), offsets by the minimum image on periodic axes, both signs at once;
then the FP64 square roots, their difference times the scale, rounded once.
Checked bit for bit against scipy's transform (oracle/unet_oracle.py
features) on grain volumes with and without periodic axes."""
import numpy as np
import pytest

from oracle import unet_oracle as UO

INF = 1 << 29


def _axis_pass(src, axis, periodic):
    n = src.shape[axis]
    q = np.arange(n)
    o = np.abs(q[:, None] - q[None, :])
    if periodic:
        o = np.minimum(o, n - o)
    o2 = (o * o).astype(np.int64)                      # [p, q]
    s = np.moveaxis(src, axis, -1)                     # [..., q]
    out = np.min(s[..., None, :] + o2, axis=-1)        # [..., p]
    return np.moveaxis(np.minimum(out, INF), -1, axis)


def features(walls, periodic, scale=0.125):
    solid = np.asarray(walls) != 0
    sq = []
    for feat in (solid, ~solid):                       # distance to solid, distance to fluid
        a = np.where(feat, 0, INF).astype(np.int64)
        a = _axis_pass(a, 2, periodic[0])              # x
        a = _axis_pass(a, 1, periodic[1])              # y
        a = _axis_pass(a, 0, periodic[2])              # z
        sq.append(a)
    x = np.empty(solid.shape + (2,), np.float32)
    x[..., 0] = solid
    x[..., 1] = (np.sqrt(sq[0].astype(np.float64)) - np.sqrt(sq[1].astype(np.float64))) * scale
    return x


def _grains(shape, frac, seed, walls_x):
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    s = ndimage.binary_dilation(rng.random(shape) < frac, iterations=2)
    if walls_x:
        s[:, :, 0] = s[:, :, -1] = True
    if not s.any():
        s[shape[0] // 3, shape[1] // 2, shape[2] // 4] = True
    return s.astype(np.int32)


@pytest.mark.parametrize("shape,frac,periodic,walls_x", [
    ((20, 12, 16), 0.01, (False, True, True), True),
    ((14, 18, 22), 0.004, (True, True, True), False),
    ((11, 7, 13), 0.02, (False, False, False), False),
    ((24, 24, 24), 0.0, (True, True, True), False)])
def test_separable_passes_match_scipy(shape, frac, periodic, walls_x):
    w = _grains(shape, frac, 7, walls_x)
    assert features(w, periodic).tobytes() == UO.features(w, periodic).tobytes()
