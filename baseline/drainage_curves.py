"""Saturation and flow-rate curves of the 256^3 drainage workload: this
library's stand-alone program (mf-lbm-cuda_gb300/lib/mflbm_main, FP32 fast
and FP64) beside the reference's own CUDA program (baseline/ref_cuda.py,
FP32 and FP64 builds), each run in its own copy of the same case folder; the
curves are read from the programs' own monitor files
(results/out1.output/saturation.dat and flowrate_time.dat,
src/Monitor.cpp:110-190: step, saturation, vol1, vol2, mass1, mass2 and
step, whole-domain / sample mean flow rates).

    python baseline/drainage_curves.py [--steps 10000] [--monitor 1000] [--size 256]
        [--programs ours_f32,ours_f64,ref_f32,ref_f64] [--json out.json]

Prints one JSON document: per program the rows of both files and the wall
time; the relative differences of saturation and sample flow rate of every
program against the reference's FP64 build at each monitor step.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "mf-lbm-cuda_gb300"))
sys.path.insert(0, str(HERE))


def case_for(size, steps, monitor):
    from mflbm import cases
    case = cases.drainage_256x256x256()
    if size != 256:
        case.keys.update({"nxGlobal": size, "nyGlobal": size, "nzGlobal": size})
    case.keys.update({"max_time_step": steps, "monitor_timer": monitor, "display_steps_timer": monitor,
                      "benchmark_cmd": 1, "ntime_visual": 10 ** 8, "ntime_animation": 10 ** 8,
                      "computation_time_timer": 10 ** 8, "block_Threads_X": 128, "block_Threads_Y": 1,
                      "block_Threads_Z": 1})
    return case


def read_dat(path):
    rows = []
    if not path.exists():
        return rows
    for line in path.read_text().splitlines():
        parts = line.split()
        if parts:
            rows.append([float(x) for x in parts])
    return rows


def run_program(name, size, steps, monitor, geometry, timeout):
    from mflbm import cases
    import ref_cuda
    case = case_for(size, steps, monitor)
    work = Path(tempfile.mkdtemp(prefix=f"mflbm_curves_{name}_"))
    try:
        cases.write_case_dir(case, str(work), geometry=geometry)
        if name.startswith("ours"):
            exe = REPO / "mf-lbm-cuda_gb300" / "lib" / "mflbm_main"
            cmd = [str(exe)] + (["--fp64"] if name.endswith("f64") else []) + [str(work)]
        else:
            cmd = [str(ref_cuda.build(name.split("_")[1]))]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, cwd=work, capture_output=True, text=True, timeout=timeout)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": f"exit {r.returncode}: {r.stdout[-1500:]} {r.stderr[-1500:]}"}
        out = work / "results" / "out1.output"
        return {"saturation": read_dat(out / "saturation.dat"), "flowrate": read_dat(out / "flowrate_time.dat"),
                "wall_s": round(wall, 2)}
    finally:
        shutil.rmtree(work, ignore_errors=True)


def compare(results, base="ref_f64"):
    """Relative differences of saturation (column 1 of saturation.dat) and of
    the sample flow rate (column 4 of flowrate_time.dat) against `base`."""
    b = results.get(base, {})
    diffs = {}
    for name, r in results.items():
        if name == base or "saturation" not in r or "saturation" not in b:
            continue
        rows = []
        for (s, sb), (f, fb) in zip(zip(r["saturation"], b["saturation"]), zip(r["flowrate"], b["flowrate"])):
            rows.append({"step": int(s[0]), "saturation_rel": abs(s[1] - sb[1]) / abs(sb[1]),
                         "flow_rate_rel": abs(f[4] - fb[4]) / max(abs(fb[4]), 1e-300)})
        diffs[name] = rows
    return diffs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--monitor", type=int, default=1000)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--programs", default="ours_f32,ours_f64,ref_f32,ref_f64")
    ap.add_argument("--timeout", type=float, default=1500.0)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    geometry = case_for(a.size, a.steps, a.monitor).geometry_bytes()
    results = {}
    for name in a.programs.split(","):
        results[name] = run_program(name, a.size, a.steps, a.monitor, geometry, a.timeout)
        print(json.dumps({name: {k: v for k, v in results[name].items() if k in ("wall_s", "error")}}),
              file=sys.stderr, flush=True)
    doc = {"lattice": [a.size] * 3, "steps": a.steps, "monitor": a.monitor, "results": results,
           "vs_ref_f64": compare(results)}
    text = json.dumps(doc)
    if a.json:
        Path(a.json).write_text(text)
    print(text)


if __name__ == "__main__":
    main()
