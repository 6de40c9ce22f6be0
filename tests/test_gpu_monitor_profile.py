"""mflbm_monitor_profile against a float64 numpy restatement of the reference's
monitor sums (src/Monitor.cpp:17-104, :277-466) on the state the library
downloads: per-slice volume, mass, flux and pressure sums, the velocity and
kinetic-energy scalars, the capillary-pressure sums, the breakthrough count
and the phase-field change between two tracking calls."""
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _expected(d, walls, params, T, shape):
    nx, ny, nz = shape
    s1 = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    s2 = (slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2))
    s4 = (slice(4, nz + 4), slice(4, ny + 4), slice(4, nx + 4))
    pdf = d["pdf"]
    f = [pdf[0, q][s1].astype(np.float64) + pdf[1, q][s1].astype(np.float64) for q in range(19)]
    rho = f[0]
    for q in range(1, 19):
        rho = rho + f[q]
    tmp = (T(0.5) * T(params.lbm_gamma) * d["curv"][s1] * d["c_norm"][s2]).astype(np.float64)
    fx = tmp * d["cn_x"][s2]
    fy = tmp * d["cn_y"][s2]
    fz = tmp * d["cn_z"][s2] + float(T(params.force_z))
    u = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] - 0.5 * fx
    v = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] - 0.5 * fy
    w = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] - 0.5 * fz
    ph = d["phi"][s4]
    fl = walls[s2] == 0
    pd = ph.astype(np.float64)
    a1, a2 = 0.5 * (1 + pd), 0.5 * (1 - pd)
    rows = {"fl1": w * a1, "fl2": w * a2, "vol1": a1, "vol2": a2, "mass1": rho * a1, "mass2": rho * a2, "pre": rho}
    prof = {n: np.where(fl, x, 0).sum(axis=(1, 2)) for n, x in rows.items()}
    scale = {n: np.where(fl, np.abs(x), 0).sum(axis=(1, 2)) for n, x in rows.items()}
    u2 = u * u + v * v + w * w
    ext = {"umax2": u2[fl].max(), "usq1": u2[fl & (ph > T(0.999))].sum(), "usq2": u2[fl & (ph < T(-0.999))].sum(),
           "pre_w": rho[fl & (ph < T(-0.99))].sum(), "pre_nw": rho[fl & (ph > T(0.99))].sum(),
           "n_w": int((fl & (ph < T(-0.99))).sum()), "n_nw": int((fl & (ph > T(0.99))).sum()),
           "breakthrough": int((fl[nz - 2] & (ph[nz - 2] > T(0))).sum())}
    return prof, scale, ext, np.where(fl, pd, 0.0)


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("kind", ["velocity_convective", "periodic_drop"])
def test_profile_matches_numpy(mflbm_lib, kind, prec):
    from mflbm import lib
    case = cases.small_case(kind)
    T = H.dtype_of(prec)
    ctx, info = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=read_dat(GOLDEN / f"{case.name}.dat"),
                               want_host_geometry=True)
    walls = info["geometry"]["walls"]
    ctx.run(1, 10)
    _, e0 = ctx.monitor_profile(track_phi=True)
    phi10 = ctx.download(["phi"])["phi"]
    ctx.run(11, 10)
    prof, ext = ctx.monitor_profile(track_phi=True)
    d = ctx.download()
    want, scale, ext_want, phi_now = _expected(d, walls, ctx.params, T, case.shape)
    for n in abi.PROFILE_ROWS:
        assert np.all(np.abs(prof[n] - want[n]) <= 1e-12 * scale[n] + 1e-300), n
    for n in ("n_w", "n_nw", "breakthrough"):
        assert ext[n] == ext_want[n], n
    for n in ("umax2", "usq1", "usq2", "pre_w", "pre_nw"):
        assert ext[n] == pytest.approx(ext_want[n], rel=1e-12, abs=1e-300), n
    # phase-field change since the previous tracking call (step 10)
    nz, ny, nx = phi_now.shape
    prev = phi10[4:nz + 4, 4:ny + 4, 4:nx + 4].astype(np.float64)
    fl = walls[2:nz + 2, 2:ny + 2, 2:nx + 2] == 0
    assert ext["dphi_max"] == np.abs(np.where(fl, phi_now - prev, 0)).max()
    assert e0["dphi_max"] == np.abs(np.where(fl, prev, 0)).max()   # first call: against zero
    ctx.close()
