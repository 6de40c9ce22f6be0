"""The drop-in acceptance run: the reference's own host program (src/main.cpp
and the other src/*.cpp of the reference, unmodified) linked against
libmflbm_refshim_f64.a + libmflbm.so in place of its CUDA files, and the
reference's own CUDA program (its kernels, compiled for this GPU), each run
on the 48 x 48 x 64 drainage workload (velocity inlet, convective outlet,
FP64, 2000 steps, monitors every 200 steps) in its own copy of the same case
folder.  The monitor files of results/out1.output must agree.

Both programs print their monitor sums with the stream's default 6
significant digits.  The reference sums serially in FP64 on the host after
copying the device state; the library's drop-in does the same (it refreshes
the host arrays at output steps), so the printed values may differ only
where FMA contraction in the two sets of kernels moves the state's last
bits: printed values must agree to 1e-5 relative.

Needs the reference's sources, which baseline/ref_cuda.py prepares under
baseline/_ref where the reference checkout exists; skipped otherwise.
"""
import subprocess
import sys
from pathlib import Path

import pytest

from mflbm import cases

REPO = Path(__file__).resolve().parent.parent
LIBDIR = REPO / "mf-lbm-cuda_gb300" / "lib"
sys.path.insert(0, str(REPO / "baseline"))
import ref_cuda  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available("f64"), reason="reference sources not prepared")]

HOST_SOURCES = ["main.cpp", "IO_multiphase.cpp", "Init_multiphase.cpp", "Misc.cpp", "Monitor.cpp",
                "Phase_gradient.cpp", "Geometry_preprocessing.cpp", "utils.cpp"]
STEPS, MONITOR = 2000, 200
FILES = ["saturation.dat", "flowrate_time.dat", "saturation_full_domain.dat", "Ca_number.dat"]


def build_dropin(tmp_path):
    """The reference's host sources (FP64 build) against the drop-in library."""
    src = ref_cuda.src_dir("f64")
    objs = []
    for s in HOST_SOURCES:
        o = tmp_path / (Path(s).stem + ".o")
        r = subprocess.run(["g++", "-O2", "-std=c++17", "-w", "-I", str(src / "includes"), "-I",
                            "/usr/local/cuda/include", "-c", str(src / "src" / s), "-o", str(o)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(str(o))
    exe = tmp_path / "mflbm_dropin_f64"
    r = subprocess.run(["g++", *objs, str(LIBDIR / "libmflbm_refshim_f64.a"), "-L", str(LIBDIR), "-lmflbm",
                        f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_in(folder, exe, case, geometry):
    cases.write_case_dir(case, str(folder), geometry=geometry)
    r = subprocess.run([str(exe)], cwd=folder, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return {f: [[float(x) for x in line.split()] for line in (folder / "results" / "out1.output" / f).read_text()
                .splitlines() if line.strip()] for f in FILES}


def test_reference_program_on_the_library_matches_the_reference(mflbm_lib, tmp_path):
    case = cases.drainage_48x48x64()
    case.keys.update({"max_time_step": STEPS, "monitor_timer": MONITOR, "ntime_visual": 10 ** 6,
                      "ntime_animation": 10 ** 6, "computation_time_timer": 10 ** 6, "display_steps_timer": 10 ** 6})
    geo = case.geometry_bytes()
    ours = run_in(tmp_path / "dropin", build_dropin(tmp_path), case, geo)
    theirs = run_in(tmp_path / "reference", ref_cuda.build("f64"), case, geo)
    for f in FILES:
        assert len(ours[f]) == len(theirs[f]) > 0, (f, len(ours[f]), len(theirs[f]))
        for a, b in zip(ours[f], theirs[f]):
            assert a[0] == b[0], (f, "step")
            for x, y in zip(a[1:], b[1:]):
                assert x == pytest.approx(y, rel=1e-5, abs=1e-12), (f, a[0], a, b)
    sat = [row[1] for row in theirs["saturation.dat"]]
    assert 0.0 < sat[0] < sat[-1] < 1.0   # the front advances: a non-trivial comparison
