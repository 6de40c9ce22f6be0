"""The stand-alone program (lib/mflbm_main) up to the point where it would
first touch the GPU: usage text and the reference's input checks
(src/IO_multiphase.cpp:16-242), which end the program with exit code 1."""
import subprocess
from pathlib import Path

import pytest

from mflbm import cases

DRIVER = Path(__file__).resolve().parent.parent / "mf-lbm-cuda_gb300" / "lib" / "mflbm_main"


def _run(folder):
    return subprocess.run([str(DRIVER), str(folder)], capture_output=True, text=True, timeout=60)


def test_usage(mflbm_lib):
    r = subprocess.run([str(DRIVER), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage: mflbm_main" in r.stdout


@pytest.mark.parametrize("change, message", [
    ({"theta": "95"}, "contact angle is larger than 90 degrees"),
    ({"iper": 1}, "X direction periodic BC enabled"),
    ({"jper": 1}, "non-slip BC applied at y = ymin or y = ymax while y direction periodic BC enabled"),
    ({"inlet_BC": 2, "outlet_BC": 1}, "Inlet pressure + outlet convective BC is not supported"),
])
def test_invalid_control_files_are_rejected(mflbm_lib, tmp_path, change, message):
    case = cases.small_case("pressure_pressure")
    case.keys.update(change)
    cases.write_case_dir(case, str(tmp_path))
    r = _run(tmp_path)
    assert r.returncode == 1
    assert message in r.stdout


def test_missing_key_and_bad_status(mflbm_lib, tmp_path):
    case = cases.small_case("pressure_pressure")
    cases.write_case_dir(case, str(tmp_path))
    ctl = tmp_path / "input" / "simulation_control.txt"
    ctl.write_text("".join(l for l in ctl.read_text().splitlines(True) if not l.startswith("RK_beta")))
    r = _run(tmp_path)
    assert r.returncode == 1 and "Couldn't find the variable named: (RK_beta)" in r.stdout
    (tmp_path / "input" / "job_status.txt").write_text("new_simulation\n")   # the reference wants the bare word
    r = _run(tmp_path)
    assert r.returncode == 1 and "Wrong simlation status" in r.stdout
