"""The C ABI library without a GPU: it loads, exports every entry point that
include/mflbm.h declares, rejects invalid input with an error code and a
message, and its host set-up functions (parameter derivation, domain walls,
inlet profile) equal the oracle bit for bit."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.abi import ptr

HEADER = Path(__file__).resolve().parent.parent / "include" / "mflbm.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mflbm_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("mflbm_create", "mflbm_step", "mflbm_run", "mflbm_upload_fields", "mflbm_download_fields",
                 "mflbm_preprocess_geometry", "mflbm_monitor_reduce", "mflbm_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(mflbm_lib):
    missing = [n for n in declared_functions() if not hasattr(mflbm_lib, n)]
    assert not missing, missing
    assert mflbm_lib.mflbm_abi_version() == 3


def test_binding_covers_every_symbol():
    from mflbm.lib import SIGNATURES
    assert sorted(SIGNATURES) == declared_functions()


CASES = [cases.small_case(k) for k in cases.SMALL_KINDS] + [cases.drainage_48x48x64(), cases.drainage_256x256x256()]


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_params_from_control_matches_oracle(mflbm_lib, case, prec):
    from mflbm import lib
    ctl = case.control(prec)
    p, d = lib.params_from_control(ctl, prec, abi.MFLBM_FAST)
    po, do = abi.Params(), abi.Derived()
    H.oracle_lib().__getattr__(f"orc_params_from_control_{H.suffix(prec)}")(C.byref(ctl), abi.MFLBM_FAST,
                                                                           C.byref(po), C.byref(do))
    assert abi.struct_dict(p) == abi.struct_dict(po)
    assert abi.struct_dict(d) == abi.struct_dict(do)


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("kind", ["velocity_convective", "pressure_pressure", "closed_contact"])
def test_walls_and_inlet_profile_match_oracle(mflbm_lib, kind, prec):
    from mflbm import lib
    case = cases.small_case(kind)
    ctl = case.control(prec)
    geo = case.geometry_bytes()
    wg = lib.set_walls(ctl, geo)
    o = H.OracleState(case, prec, geometry=geo)
    assert np.array_equal(wg, o.a["walls_global"])
    w = lib.inlet_profile(ctl, prec)
    assert w.tobytes() == o.a["W_in"].tobytes()


def test_inlet_profile_48x48x64_matches_oracle(mflbm_lib):
    from mflbm import lib
    case = cases.drainage_48x48x64()
    for prec in (abi.MFLBM_FP32, abi.MFLBM_FP64):
        ctl = case.control(prec)
        w = lib.inlet_profile(ctl, prec)
        ref = abi.Layout(*case.shape).empty("plane1", H.dtype_of(prec))
        H.oracle_lib().__getattr__(f"orc_inlet_profile_{H.suffix(prec)}")(C.byref(ctl), ptr(ref))
        assert w.tobytes() == ref.tobytes()
        # the duct profile carries the prescribed mean velocity over the open section
        assert abs(w.mean() * w.size / ((case.shape[0] - 2) * (case.shape[1] - 2)) - 1e-4) < 2e-6


def test_invalid_input_is_rejected_with_a_message(mflbm_lib):
    from mflbm import lib
    case = cases.small_case("velocity_convective")
    ctl = case.control(abi.MFLBM_FP64)
    ctl.theta = 120.0
    with pytest.raises(lib.MflbmError, match="contact angle"):
        lib.params_from_control(ctl, abi.MFLBM_FP64, abi.MFLBM_FAST)
    ctl = case.control(abi.MFLBM_FP64)
    ctl.domain_wall_status_x_min = 0
    with pytest.raises(lib.MflbmError, match="x must be walled"):
        lib.params_from_control(ctl, abi.MFLBM_FP64, abi.MFLBM_FAST)
    p, _ = lib.params_from_control(case.control(abi.MFLBM_FP64), abi.MFLBM_FP64, abi.MFLBM_FAST)
    p.precision = 3
    h = C.c_void_p()
    assert mflbm_lib.mflbm_create(C.byref(p), C.byref(h)) == -1
    assert b"precision" in mflbm_lib.mflbm_last_error()
    p.precision = abi.MFLBM_FP64
    p.nx = 2000
    assert mflbm_lib.mflbm_create(C.byref(p), C.byref(h)) == -1
    assert not h.value


def test_warm_start_entries_reject_bad_arguments_before_device_work(mflbm_lib):
    """mflbm_unet_features and mflbm_init_flow_predicted check their
    arguments on the host (no device is touched for these calls)."""
    import numpy as np
    from mflbm.abi import ptr
    x = np.empty((4, 4, 4, 2), np.float32)
    fluid = np.zeros((4, 4, 4), np.int32)
    assert mflbm_lib.mflbm_unet_features(None, 4, 4, 4, 0, C.c_float(0.125), ptr(x)) == -1
    assert b"null argument" in mflbm_lib.mflbm_last_error()
    assert mflbm_lib.mflbm_unet_features(ptr(fluid), 0, 4, 4, 0, C.c_float(0.125), ptr(x)) == -1
    assert b"extents" in mflbm_lib.mflbm_last_error()
    assert mflbm_lib.mflbm_unet_features(ptr(fluid), 4, 4, 4, 0, C.c_float(0.125), ptr(x)) == -1
    assert b"both solid and fluid" in mflbm_lib.mflbm_last_error()
    assert mflbm_lib.mflbm_unet_features(ptr(fluid), 4096, 4096, 4096, 0, C.c_float(0.125), ptr(x)) == -1
    assert b"2^31" in mflbm_lib.mflbm_last_error()
    y = np.zeros(4, np.float32)
    assert mflbm_lib.mflbm_init_flow_predicted(None, ptr(y), 1.0 / 6.0, 1e-4, ptr(y), 1) == -1
    assert b"null argument" in mflbm_lib.mflbm_last_error()
