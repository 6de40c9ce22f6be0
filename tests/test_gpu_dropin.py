"""The drop-in entry points driven the way the reference's main() drives them
(src/main.cpp:97-99, 145-147): globals hold the start-up state in the
reference layouts, initialization_GPU() / copyConstantData() upload it, and
main_iteration_kernel_GPU() runs each time step with the host arrays
refreshed at output steps.  Strict flavour: bit-identical to the oracle."""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parent.parent
LIBDIR = REPO / "mf-lbm-cuda_gb300" / "lib"
GOLDEN = REPO / "tests" / "golden"


def build_host(tmp_path, prec):
    out = tmp_path / f"dropin_host_{prec}.so"
    define = ["-DMFLBM_REF_DOUBLE"] if prec == "f64" else []
    r = subprocess.run(["g++", "-shared", "-fPIC", "-O1", *define, str(REPO / "tests" / "dropin" / "host_globals.cpp"),
                        "-Wl,--whole-archive", str(LIBDIR / f"libmflbm_refshim_{prec}.a"), "-Wl,--no-whole-archive",
                        "-L", str(LIBDIR), "-lmflbm", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return C.CDLL(str(out))


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("kind", ["velocity_convective", "pressure_pressure"])
def test_reference_entry_points_bit_exact(mflbm_lib, tmp_path, kind, prec):
    os.environ["MFLBM_FP_MODE"] = "strict"
    lib = build_host(tmp_path, H.suffix(prec))
    case = cases.small_case(kind)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    o = H.OracleState(case, prec, geometry=geo)
    # host arrays in the reference layouts, owned here, pointed to by the globals
    host = {n: o.a[n].copy() for n in ("pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "W_in",
                                       "f_convec_bc", "g_convec_bc", "phi_convec_bc", "walls", "walls_type",
                                       "s_nx", "s_ny", "s_nz")}
    TP = C.c_float if prec == abi.MFLBM_FP32 else C.c_double
    for n, a in host.items():
        C.c_void_p.in_dll(lib, n).value = a.ctypes.data
    ctl = o.control
    for n in ("nxGlobal", "nyGlobal", "nzGlobal"):
        C.c_longlong.in_dll(lib, n).value = getattr(ctl, n)
    for n in ("iper", "jper", "kper", "domain_wall_status_x_min", "domain_wall_status_x_max",
              "domain_wall_status_y_min", "domain_wall_status_y_max", "domain_wall_status_z_min",
              "domain_wall_status_z_max", "inlet_BC", "outlet_BC", "porous_plate_cmd", "Z_porous_plate"):
        C.c_int.in_dll(lib, n).value = getattr(ctl, n)
    p = o.params
    for g, v in (("lbm_gamma", p.lbm_gamma), ("lbm_beta", p.lbm_beta), ("cos_theta", p.cos_theta),
                 ("phi_inlet", p.phi_inlet), ("sa_inject", p.sa_inject), ("la_nui2", p.la_nui2),
                 ("force_z", p.force_z), ("uin_avg", p.uin_avg), ("rho_in", p.rho_in), ("rho_out", p.rho_out),
                 ("relaxation", p.relaxation), ("la_nui1", p.la_nui1)):
        TP.in_dll(lib, g).value = v
    nsteps = 12
    for n in ("ntime_monitor", "ntime_animation", "ntime_visual", "ntime_clock_sum"):
        C.c_int.in_dll(lib, n).value = nsteps
    getattr(lib, "_Z18initialization_GPUv")()
    getattr(lib, "_Z16copyConstantDatav")()
    for nt in range(1, nsteps + 1):
        C.c_int.in_dll(lib, "ntime").value = nt
        getattr(lib, "_Z25main_iteration_kernel_GPUv")()
    o.run(nsteps)
    for n in ("pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv"):
        assert host[n].tobytes() == o.a[n].tobytes(), n
    getattr(lib, "_Z24MemAllocate_geometry_GPUi")(2)
    getattr(lib, "_Z21MemAllocate_multi_GPUi")(2)
