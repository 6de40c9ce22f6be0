"""mflbm_upload_fields / mflbm_download_fields with page-locked host buffers.

With page-locked (pinned) host memory the upload's population relayout
kernel reads the caller's reference-layout array directly over the host
link; with ordinary memory the copy goes through the device staging buffer.
Both paths must move exactly the same bytes: a state uploaded from pinned memory
and stepped must equal the same state uploaded from ordinary memory, bit for
bit, and a download into pinned buffers must equal a download into ordinary
arrays.
"""
from pathlib import Path

import numpy as np
import pytest

from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ("pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "f_convec_bc", "g_convec_bc", "phi_convec_bc")


def _pinned_like(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.float32, pin_memory=True)
    out = t.numpy().reshape(a.shape)
    out[...] = a
    return t, out


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
def test_pinned_and_ordinary_host_buffers_move_the_same_bytes(mflbm_lib, prec):
    from mflbm import lib
    case = cases.small_case("velocity_convective")
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, info = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=geo)
    ctx.run(1, 6)
    state = ctx.download()
    keep = []   # the pinned tensors own the buffers
    pinned = {}
    for n, a in state.items():
        t, p = _pinned_like(a)
        keep.append(t)
        pinned[n] = p
    # download into pinned buffers == download into ordinary arrays
    into = {}
    for n, a in state.items():
        t, p = _pinned_like(np.zeros_like(a))
        keep.append(t)
        into[n] = p
    ctx.download(out=into)
    for n in state:
        assert into[n].tobytes() == state[n].tobytes(), n
    # upload from pinned, step; upload the same from ordinary memory, step
    results = []
    for src in (pinned, {n: np.array(a) for n, a in state.items()}):
        c2, _ = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=geo)
        c2.upload_fields(W_in=info["W_in"], **src)
        c2.run(7, 4)
        results.append(c2.download())
        c2.close()
    for n in NAMES:
        assert results[0][n].tobytes() == results[1][n].tobytes(), n
    ctx.close()
