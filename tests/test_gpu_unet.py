"""The U-Net's tensor-core convolutions, their gradients and the whole
network's gradients against the CPU restatement (oracle/unet_oracle.py),
plus the warm-start equilibrium fill (mflbm_init_flow).

Tolerances: convolution outputs and weight gradients are FP32 sums of exact
BF16 products, so they agree with the FP64 sums to 2e-5 of the sum of
absolute terms; data gradients are rounded to BF16 (2^-8 relative) on both
sides and may differ by one BF16 step.  Whole-network gradients pass through
BF16 activations on both sides; single rounding flips propagate, so each
layer's gradient is compared by relative L2 error (<= 3e-2) and the loss to
1e-3."""
import numpy as np
import pytest

from mflbm import unet
from oracle import unet_oracle as UO

pytestmark = pytest.mark.gpu


def _bf(a):
    return UO.bf16(np.asarray(a, np.float32)).astype(np.float64)


@pytest.mark.parametrize("shape,cin,cout,relu", [((5, 7, 9), 16, 16, False), ((4, 6, 10), 48, 32, True),
                                                 ((3, 5, 6), 64, 128, False), ((6, 6, 6), 96, 32, True),
                                                 ((4, 4, 8), 192, 64, False), ((16, 16, 12), 16, 16, True)])
def test_conv_forward_and_gradients_match_oracle(mflbm_lib, shape, cin, cout, relu):
    _check_conv(shape, cin, cout, relu)


# Volumes with at least one halo tile (8 x 16 x tz voxels) per multiprocessor
# of a GB300 (152): the halo-tiled kernel (unet_halo.cuh) serves the forward
# pass and the data gradient here, with partial tiles at the x, y and z ends;
# tz = 4 for (62, 60, 36) with 16 -> 16, tz = 1 elsewhere; 48 -> 16 has six
# channel groups, its data gradient 48 output channels.
@pytest.mark.parametrize("shape,cin,cout,relu", [((62, 60, 36), 16, 16, True), ((40, 48, 36), 48, 16, False),
                                                 ((40, 30, 20), 32, 32, True), ((34, 32, 24), 16, 32, False)])
def test_halo_conv_forward_and_gradients_match_oracle(mflbm_lib, shape, cin, cout, relu):
    _check_conv(shape, cin, cout, relu)


@pytest.mark.parametrize("shape,cin,cout", [((5, 7, 9), 16, 16), ((40, 30, 20), 32, 32)], ids=["gather", "halo"])
def test_stage_wait_that_runs_out_is_reported(mflbm_lib, shape, cin, cout):
    """A bound of 0 polls makes every pipeline-stage wait of the tensor-core
    convolutions run out (the gather kernels and, at the second shape, the
    halo-tiled kernel): the call fails with the time-out error, the kernels
    still wait (with the full bound) for their copies and MMAs before freeing
    tensor memory, and with the default bound the next call is exact again."""
    from mflbm import lib
    L = lib.load()
    rng = np.random.default_rng(5)
    D, H, W = shape
    x = rng.normal(size=(D, H, W, cin)).astype(np.float32)
    w = (rng.normal(size=(cout, 27, cin)) / np.sqrt(27 * cin)).astype(np.float32)
    b = rng.normal(size=cout).astype(np.float32)
    gy = rng.normal(size=(D, H, W, cout)).astype(np.float32)
    lib.check(L.mflbm_unet_set_wait_limit(0), "mflbm_unet_set_wait_limit")
    try:
        with pytest.raises(lib.MflbmError, match="timed out"):
            unet.conv_check(x, w, b, gy, relu=False)
    finally:
        lib.check(L.mflbm_unet_set_wait_limit(1 << 20), "mflbm_unet_set_wait_limit")
    _check_conv(shape, cin, cout, False)


def _check_conv(shape, cin, cout, relu):
    rng = np.random.default_rng(cin + cout)
    D, H, W = shape
    x = rng.normal(size=(D, H, W, cin)).astype(np.float32)
    w = (rng.normal(size=(cout, 27, cin)) / np.sqrt(27 * cin)).astype(np.float32)
    b = rng.normal(size=cout).astype(np.float32)
    gy = rng.normal(size=(D, H, W, cout)).astype(np.float32)
    y, gx, gw, gb = unet.conv_check(x, w, b, gy, relu=relu)
    xb, wb, gyb = _bf(x), _bf(w), _bf(gy)
    ref = UO.conv(xb, wb, b.astype(np.float64))
    scale = UO.conv(np.abs(xb), np.abs(wb))
    if relu:
        ref = np.maximum(ref, 0)
    assert np.all(np.abs(y - ref) <= 2e-5 * scale + 1e-6)
    gw_ref, gb_ref = UO.conv_wgrad(xb, gyb)
    gw_scale, _ = UO.conv_wgrad(np.abs(xb), np.abs(gyb))
    assert np.all(np.abs(gw - gw_ref) <= 2e-5 * gw_scale + 1e-6)
    assert np.allclose(gb, gb_ref, rtol=1e-5, atol=1e-4)
    gx_ref = UO.conv_dgrad(gyb, wb)
    gx_scale = UO.conv_dgrad(np.abs(gyb), np.abs(wb))
    assert np.all(np.abs(gx - gx_ref) <= 2 ** -8 * np.abs(gx_ref) + 2e-5 * gx_scale + 1e-6)


# 16^3: every convolution on the gather kernels; 64^3 (the training size of
# the warm-start study): levels 0 and 1 on the halo-tiled kernels (at least
# one tile per multiprocessor), forward and data gradients.
@pytest.mark.parametrize("D", [16, 64])
def test_network_gradients_match_oracle(mflbm_lib, D):
    rng = np.random.default_rng(7)
    net = unet.UNet(D, D, D, seed=3)
    assert net.n_params == UO.param_count()
    p = UO.init_params(5)
    net.set_params(p)
    assert np.array_equal(net.get_params(), p)
    x = np.zeros((D, D, D, 2), np.float32)
    x[..., 0] = rng.random((D, D, D)) < 0.4
    x[..., 1] = rng.normal(size=(D, D, D))
    t = rng.normal(size=(D, D, D, 4)).astype(np.float32)
    m = (x[..., 0] == 0).astype(np.float32)
    loss, g = net.gradients(x, t, m)
    loss_ref, g_ref = UO.loss_and_gradients(p, x, t, m)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    o = 0
    errs = []
    for li, (ci, co, _) in enumerate(UO.layer_shapes()):
        n = co * 27 * ci + co
        a, r = g[o:o + n].astype(np.float64), g_ref[o:o + n].astype(np.float64)
        o += n
        err = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
        errs.append(err)
    y = net.forward(x)
    y_ref, _, _ = UO.forward(p, x)
    print("layer gradient errors", [round(e, 4) for e in errs],
          "forward", float(np.max(np.abs(y - y_ref)) / np.max(np.abs(y_ref))))
    assert max(errs) <= 3e-2, errs
    assert np.max(np.abs(y - y_ref)) <= 2e-2 * np.max(np.abs(y_ref))
    net.close()


def test_training_reduces_the_loss(mflbm_lib):
    D = 16
    rng = np.random.default_rng(11)
    net = unet.UNet(D, D, D, seed=1)
    data = []
    for s in range(4):
        x = np.zeros((D, D, D, 2), np.float32)
        x[..., 0] = rng.random((D, D, D)) < 0.3
        x[..., 1] = rng.normal(size=(D, D, D))
        t = np.stack([x[..., 1], -x[..., 1], 0.5 * x[..., 0], np.roll(x[..., 1], 1, 0)], -1).astype(np.float32)
        data.append((x, t, np.ones((D, D, D), np.float32)))
    first = np.mean([net.gradients(*d)[0] for d in data])
    losses, _ = unet.train(net, data, epochs=60, lr=3e-3, lr_end=3e-4)
    assert losses[-1] < 0.5 * first and losses[-1] < losses[0], (first, losses)
    net.close()


def test_init_flow_fills_the_equilibrium(mflbm_lib):
    from mflbm import abi, cases, lib
    case = cases.permeability_sample(16, 0.6, 5)
    ctx, info = lib.setup_case(case, abi.MFLBM_FP64, abi.MFLBM_STRICT, want_host_geometry=True)
    L = ctx.L
    shp = (L.nz + 2, L.ny + 2, L.nx + 2)
    cold = ctx.download(("pdf",))["pdf"].reshape(2, 19, *shp)
    ctx.init_flow()
    # rest state: bit-identical to the cold start on the fluid nodes (solid nodes
    # hold the start-up wetting extrapolation of phi, which the cold start's
    # fill precedes)
    walls = info["geometry"]["walls"].reshape(L.nz + 4, L.ny + 4, L.nx + 4)[1:L.nz + 3, 1:L.ny + 3, 1:L.nx + 3]
    rest = ctx.download(("pdf",))["pdf"].reshape(2, 19, *shp)
    assert np.array_equal(rest[:, :, walls == 0], cold[:, :, walls == 0])
    rng = np.random.default_rng(2)
    rho = 1 + 1e-3 * rng.normal(size=shp)
    u, v, w = (1e-2 * rng.normal(size=shp) for _ in range(3))
    ctx.init_flow(rho, u, v, w)
    pdf = ctx.download(("pdf",))["pdf"].reshape(2, 19, *shp)
    phi = ctx.download(("phi",))["phi"].reshape(L.nz + 8, L.ny + 8, L.nx + 8)[3:L.nz + 5, 3:L.ny + 5, 3:L.nx + 5]
    wq = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    usq = u * u + v * v + w * w
    for gg, r in enumerate((rho * (1 + phi) * 0.5, rho * (1 - phi) * 0.5)):
        for q in range(19):
            cu = unet.EX[q] * u + unet.EY[q] * v + unet.EZ[q] * w
            ref = r * wq[q] * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
            assert np.allclose(pdf[gg, q], ref, rtol=1e-13, atol=1e-16)
    # the MRT-consistent fill: same mass and momentum per node, energy-square
    # moment of the total on the collision's equilibrium (-475/63 j^2)
    ctx.init_flow(rho, u, v, w, mrt=True)
    pm = ctx.download(("pdf",))["pdf"].reshape(2, 19, *shp)
    for gg in range(2):
        assert np.allclose(pm[gg].sum(0), pdf[gg].sum(0), rtol=1e-13, atol=1e-15)
        for E in (unet.EX, unet.EY, unet.EZ):
            assert np.allclose(np.tensordot(E, pm[gg], 1), np.tensordot(E, pdf[gg], 1), rtol=1e-12, atol=1e-15)
    f = pm[0] + pm[1]
    b = np.array([12.0] + [-4.0] * 6 + [1.0] * 12)
    j2 = sum((rho * c) ** 2 for c in (u, v, w))
    assert np.allclose(np.tensordot(b, f, 1), -475.0 / 63.0 * j2, rtol=1e-9, atol=1e-13)
    ctx.close()



def _grains(shape, frac, seed, walls_x=False):
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    s = ndimage.binary_dilation(rng.random(shape) < frac, iterations=2)
    if walls_x:
        s[:, :, 0] = s[:, :, -1] = True
    return s.astype(np.int32)


# Network inputs on the device (mflbm_unet_features) against scipy's exact
# distance transform: bit-identical (both take the FP64 square root of the
# same integer squared distance, scale by a power of two and round once).
# The lone-grain cases have fluid voxels more than half a period from the
# grain, so the minimum image decides their distance.
@pytest.mark.parametrize("shape,frac,periodic,walls_x", [
    ((32, 16, 24), 0.01, (False, True, True), True),
    ((20, 28, 36), 0.004, (True, True, True), False),
    ((17, 9, 23), 0.02, (False, False, False), False),
    ((40, 40, 40), 0.0, (True, True, True), False),
    ((40, 36, 44), 0.0, (False, True, True), True)])
def test_features_match_oracle(mflbm_lib, shape, frac, periodic, walls_x):
    w = _grains(shape, frac, 7, walls_x)
    if w.sum() == 0:
        w[shape[0] // 3, shape[1] // 2, shape[2] // 4] = 1   # one lone grain voxel
    nz, ny, nx = shape
    x = unet.features(w, (nx, ny, nz), periodic)
    ref = UO.features(w, periodic)
    assert x.tobytes() == ref.tobytes()


def test_features_reject_uniform_geometry(mflbm_lib):
    from mflbm import lib
    with pytest.raises(lib.MflbmError, match="both solid and fluid"):
        unet.features(np.zeros((8, 8, 8), np.int32), (8, 8, 8))


def _host_fields(y, walls_global, shape, nu, g, scales):
    """The warm-start fields of a normalised prediction, restated in numpy
    (periodic y and z halos, resting x halos): the formula of
    mflbm_init_flow_predicted, in FP32 (numpy keeps a float32 array float32
    against Python scalars, which it rounds to float32)."""
    nx, ny, nz = shape
    solid = (np.asarray(walls_global).reshape(nz, ny, nx) != 0)
    phys = y * np.asarray(scales, np.float32)
    c = g / nu
    fields = [np.where(solid, 1.0, 1.0 + 3.0 * g * phys[..., 3])]
    fields += [np.where(solid, 0.0, phys[..., a] * c) for a in range(3)]

    def halo(f, fill):
        p = np.pad(f, ((1, 1), (1, 1), (0, 0)), mode="wrap")
        return np.pad(p, ((0, 0), (0, 0), (1, 1)), constant_values=fill)
    return [halo(fields[0], 1.0)] + [halo(f, 0.0) for f in fields[1:]]


# The device fill from a prediction equals the host formula followed by
# mflbm_init_flow(_mrt), byte for byte, in FP32 and FP64 (a 24 x 24 x 32
# permeability sample, periodic in y and z).
@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("mrt", [False, True])
def test_predicted_fill_matches_host_formula(mflbm_lib, precision, mrt):
    from mflbm import abi, cases, lib
    prec = abi.MFLBM_FP32 if precision == "f32" else abi.MFLBM_FP64
    case = cases.permeability_sample(16, 0.55, 11, body_force=1e-4)
    case.keys.update({"nxGlobal": 24, "nyGlobal": 24, "nzGlobal": 32})
    nx, ny, nz = case.shape
    rng = np.random.default_rng(4)
    y = rng.normal(size=(nz, ny, nx, 4)).astype(np.float32)
    scales = np.array([0.8, 0.8, 2.1, 6.0], np.float32)
    nu, g = 1.0 / 6.0, 1e-4
    dev, info = lib.setup_case(case, prec, abi.MFLBM_FAST)
    host, _ = lib.setup_case(case, prec, abi.MFLBM_FAST)
    dev.init_flow_predicted(y, nu, g, scales, mrt=mrt)
    host.init_flow(*_host_fields(y, info["walls_global"], (nx, ny, nz), nu, g, scales), mrt=mrt)
    a, b = dev.download(("pdf",))["pdf"], host.download(("pdf",))["pdf"]
    assert a.tobytes() == b.tobytes()
    dev.close()
    host.close()
