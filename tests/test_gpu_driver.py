"""The stand-alone program (lib/mflbm_main) on a small case, strict flavour:
the files it writes along the run (start-up and animation phase VTK, full
VTK, final checkpoint) are byte-identical to the oracle writers' files for
the oracle's state at the same steps, the monitor files hold the FP64
monitor sums of those states, the job status follows the reference's end of
run, and a restart from the written checkpoint reaches the oracle's state
(re-running the saved step, as the reference's main loop does)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parent.parent
DRIVER = REPO / "mf-lbm-cuda_gb300" / "lib" / "mflbm_main"
GOLDEN = REPO / "tests" / "golden"
TIMERS = {"max_time_step": 40, "monitor_timer": 10, "monitor_profile_timer_ratio": 2, "ntime_animation": 20,
          "ntime_visual": 40, "computation_time_timer": 20, "display_steps_timer": 20, "benchmark_cmd": 0}


def _drive(folder, prec):
    args = [str(DRIVER), "--strict"] + (["--fp64"] if prec == abi.MFLBM_FP64 else []) + [str(folder)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r


def _saturation_line(o, nt, T):
    """The values of saturation.dat for the oracle state (FP64 sums)."""
    nx, ny, nz = o.case.shape
    k = o.case.control_keys()
    nin, nout = int(k["n_exclude_inlet"]), int(k["n_exclude_outlet"])
    s1 = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    s2 = (slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2))
    s4 = (slice(4, nz + 4), slice(4, ny + 4), slice(4, nx + 4))
    a = o.a
    rho = sum(a["pdf"][0, q][s1].astype(np.float64) + a["pdf"][1, q][s1].astype(np.float64) for q in range(19))
    fl = a["walls"][s2] == 0
    ph = a["phi"][s4].astype(np.float64)
    a1, a2 = np.where(fl, 0.5 * (1 + ph), 0), np.where(fl, 0.5 * (1 - ph), 0)
    w = slice(nin, nz - nout)
    v1, v2 = a1[w].sum(), a2[w].sum()
    m1, m2 = (rho * a1)[w].sum(), (rho * a2)[w].sum()
    return [nt] + [float(T(x)) for x in (v1 / (v1 + v2), v1, v2, m1, m2)]


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
def test_driver_run_and_restart(mflbm_lib, tmp_path, prec):
    T = H.dtype_of(prec)
    case = cases.small_case("velocity_convective")
    case.keys.update(TIMERS)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    cases.write_case_dir(case, str(tmp_path), geometry=geo)
    _drive(tmp_path, prec)
    assert (tmp_path / "job_status.txt").read_text() == "simulation_reached_max_step\n"
    res = tmp_path / "results"
    ff = res / "out3.field_data"
    o = H.OracleState(case, prec, geometry=geo)
    ref = tmp_path / "oracle"
    ref.mkdir()

    def same(path, vtk_type, nt):
        o._f("write_vtk")(*([H.C.byref(o.params)] + [H.ptr(o.a[n]) for n in ("walls", "pdf", "phi", "cn_x", "cn_y",
                                                                            "cn_z", "c_norm", "curv")]
                            + [vtk_type, 0, str(ref / "x.vtk").encode()]))
        assert H.file_digest(path) == H.file_digest(ref / "x.vtk"), (path.name, nt)

    same(ff / "phase_distribution" / "small_0000000001.vtk", 2, 1)        # written before the first step
    o.write_outputs(ref, 0)
    assert H.file_digest(ff / "walls_bin.vtk") == H.file_digest(ref / "walls_bin.vtk")
    sat = [list(map(float, l.split())) for l in (res / "out1.output" / "saturation.dat").read_text().splitlines()]
    assert [int(l[0]) for l in sat] == [10, 20, 30, 40]
    for nt in (10, 20, 30, 40):
        o.run(nt - o.ntime + 1)
        want = _saturation_line(o, nt, T)
        got = sat[[int(l[0]) for l in sat].index(nt)]
        assert got == pytest.approx(want, rel=1e-5), nt
        if nt in (20, 40):
            same(ff / "phase_distribution" / f"small_{nt:010d}.vtk", 2, nt)
    same(ff / "full_flow_field" / "full_flow_field_0000000040.vtk", 1, 40)
    o.run(1)                                                              # the loop's last step, 41
    same(ff / "full_flow_field" / "full_flow_field_0000000041.vtk", 1, 41)
    o.write_outputs(ref, 41)
    assert H.file_digest(res / "out2.checkpoint" / "id0000") == H.file_digest(ref / "checkpoint")
    for name in ("Ca_number.dat", "flowrate_time.dat", "saturation_full_domain.dat", "pre.dat", "time.dat"):
        assert (res / "out1.output" / name).exists(), name
    assert (res / "out1.output" / "profile" / "monitor 00000020").exists()

    # restart: the checkpoint stores step 42; the loop resumes at 41 and runs 10 more steps (41 .. 51)
    (tmp_path / "input" / "job_status.txt").write_text("continue_simulation")
    ctl = tmp_path / "input" / "simulation_control.txt"
    ctl.write_text(ctl.read_text().replace("max_time_step 40\n", "max_time_step 10\n"))
    _drive(tmp_path, prec)
    o.ntime = 41
    o.run(11)
    o.write_outputs(ref, 51)
    assert H.file_digest(res / "out2.checkpoint" / "id0000") == H.file_digest(ref / "checkpoint")
