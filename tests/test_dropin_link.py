"""Drop-in at the symbol level: the reference's own host program (src/main.cpp
and the other src/*.cpp of the reference checkout, unmodified) links against
libmflbm_refshim_f32.a + libmflbm.so in place of the reference's
main_iteration_GPU.cu and Init_multiphase_GPU.cu.  Needs the reference
checkout; outputs go to a temporary folder."""
import subprocess
from pathlib import Path

import pytest

from oracle import build as obuild

REPO = Path(__file__).resolve().parent.parent
LIBDIR = REPO / "mf-lbm-cuda_gb300" / "lib"

pytestmark = pytest.mark.skipif(not obuild.ref_available(), reason="reference checkout not present")

HOST_SOURCES = ["main.cpp", "IO_multiphase.cpp", "Init_multiphase.cpp", "Misc.cpp", "Monitor.cpp",
                "Phase_gradient.cpp", "Geometry_preprocessing.cpp", "utils.cpp"]


def test_reference_host_program_links_against_the_dropin(mflbm_lib, tmp_path):
    ref = obuild.REFERENCE
    objs = []
    for s in HOST_SOURCES:
        o = tmp_path / (Path(s).stem + ".o")
        r = subprocess.run(["g++", "-O1", "-std=c++17", "-w", "-I", str(ref / "includes"), "-I",
                            str(obuild.CUDA_INC), "-c", str(ref / "src" / s), "-o", str(o)], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        objs.append(str(o))
    exe = tmp_path / "mflbm_reference_host"
    r = subprocess.run(["g++", *objs, str(LIBDIR / "libmflbm_refshim_f32.a"), "-L", str(LIBDIR), "-lmflbm",
                        f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-C", str(exe)], capture_output=True, text=True).stdout
    for sym in ("main_iteration_kernel_GPU()", "initialization_GPU()", "copyConstantData()",
                "MemAllocate_geometry_GPU(int)", "MemAllocate_multi_GPU(int)"):
        assert sym in nm, sym
