"""Recipe for the reference's own CUDA program on the GB300 (measurement only).

The reference (MF-LBM-CUDA) is timed as shipped: its unmodified kernels,
launch sequence and host program, compiled for sm_103a, running the 256^3
drainage workload from its own control file.  Nothing of this library is on
that path.  Two documented patches are applied to a copy of the sources
(never to the checkout, never committed):

  1. src/Init_multiphase_GPU.cu: the print of cudaDeviceProp::clockRate is
     dropped.  CUDA 13 removed that field, so the unpatched file does not
     compile; the line only prints the clock.
  2. src/Init_multiphase_GPU.cu: the device allocations of walls_d, cn_x_d,
     cn_y_d, cn_z_d and c_norm_d get one element more than
     mem_size_s2_int / mem_size_s2_TP (walls_d's extra element is set to 0).
     normalDirectionsOfInterfaces (src/main_iteration_GPU.cu:757-807) runs
     i up to nxGlobal+3 (guard `i < nxGlobal_d + 4`, :764) on the s2 layout,
     whose x range ends at nxGlobal+2; i_s2 aliases that column into the next
     row, and at the last (j, k) row the kernel writes cn_x/y/z and c_norm
     and reads walls one element past the end of each allocation.  With one
     more element the accesses stay inside the buffers; no kernel, launch or
     result changes.
The FP64 build additionally selects the reference's own precision switch
(includes/solver_precision.h: PRECISION (DOUBLE_PRECISION)).

Steps:
  prepare()  (where the reference checkout exists): copy src/ and includes/
             into baseline/_ref/cuda_{f32,f64}/ and apply the patches there.
  build(p)   nvcc for sm_103a (one command over the copied sources; not the
             reference's Makefile): baseline/_ref/cuda_<p>/MF_LBM_CUDA.
  run(p, steps)  writes the reference's input folder for the workload in a
             temporary directory, runs the program there and parses its
             MLUPS lines (src/main.cpp:191-199, 267-271).

    python baseline/ref_cuda.py prepare
    python baseline/ref_cuda.py run --precision f32 --steps 1000
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
# The reference checkout: $MFLBM_REFERENCE, else a "reference" folder beside
# this repository's folder (only prepare() reads it).
REFERENCE = Path(os.environ.get("MFLBM_REFERENCE", str(REPO.parent / "reference")))

OUT = HERE / "_ref"
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (file, text in the reference, replacement, reason); each text must occur once
PATCHES = [
    ("src/Init_multiphase_GPU.cu",
     '    cout << "  Clock frequencey: " << props.clockRate / 1e3 << " MHz" << endl;\n', "",
     "cudaDeviceProp::clockRate is gone in CUDA 13 (print only)"),
    ("src/Init_multiphase_GPU.cu",
     "cudaErrorCheck(cudaMalloc(&walls_d, mem_size_s2_int));",
     "cudaErrorCheck(cudaMalloc(&walls_d, mem_size_s2_int + sizeof(int))); "
     "cudaErrorCheck(cudaMemset((char*)walls_d + mem_size_s2_int, 0, sizeof(int)));",
     "normalDirectionsOfInterfaces reads walls one element past the end"),
] + [
    ("src/Init_multiphase_GPU.cu",
     f"cudaErrorCheck(cudaMalloc(&{a}, mem_size_s2_TP));",
     f"cudaErrorCheck(cudaMalloc(&{a}, mem_size_s2_TP + sizeof(T_P)));",
     f"normalDirectionsOfInterfaces writes {a} one element past the end")
    for a in ("cn_x_d", "cn_y_d", "cn_z_d", "c_norm_d")
]
PRECISION_SWITCH = ("includes/solver_precision.h", "#define PRECISION (SINGLE_PRECISION)",
                    "#define PRECISION (DOUBLE_PRECISION)", "FP64 build")


def src_dir(precision: str) -> Path:
    return OUT / f"cuda_{precision}"


def binary(precision: str) -> Path:
    return src_dir(precision) / "MF_LBM_CUDA"


def available(precision: str = "f32") -> bool:
    return (src_dir(precision) / "src" / "main.cpp").exists()


def prepare() -> list:
    """Patched copies of the reference's sources under baseline/_ref/."""
    if not (REFERENCE / "src" / "main_iteration_GPU.cu").exists():
        raise FileNotFoundError(f"reference checkout not found at {REFERENCE}")
    made = []
    for precision in ("f32", "f64"):
        dst = src_dir(precision)
        if dst.exists():
            shutil.rmtree(dst)
        for sub in ("src", "includes"):
            shutil.copytree(REFERENCE / sub, dst / sub)
        patches = PATCHES + ([PRECISION_SWITCH] if precision == "f64" else [])
        for rel, old, new, _ in patches:
            p = dst / rel
            text = p.read_text(encoding="utf-8-sig")
            if text.count(old) != 1:
                raise RuntimeError(f"patch target not found exactly once in {rel}: {old!r}")
            p.write_text(text.replace(old, new), encoding="utf-8")
        made.append(dst)
    return made


def build(precision: str = "f32", force: bool = False) -> Path:
    out = binary(precision)
    if out.exists() and not force:
        return out
    d = src_dir(precision)
    srcs = sorted(str(p.relative_to(d)) for p in list((d / "src").glob("*.cu")) + list((d / "src").glob("*.cpp")))
    cmd = [NVCC, *ARCH, "-std=c++17", "-rdc=true", "-O3", "-lineinfo", "-Xcompiler", "-O3", "-I", "includes",
           *srcs, "-o", "MF_LBM_CUDA", "-lcudart"]
    r = subprocess.run(cmd, cwd=d, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return out


def drainage_case(size: int, steps: int, display: int):
    sys.path.insert(0, str(REPO / "mf-lbm-cuda_gb300"))
    from mflbm import cases
    case = cases.drainage_256x256x256()
    if size != 256:
        case.keys.update({"nxGlobal": size, "nyGlobal": size, "nzGlobal": size})
    # timers: no output, monitor or host copy inside the loop; MLUPS printed every `display` steps
    case.keys.update({"max_time_step": steps, "display_steps_timer": display, "benchmark_cmd": 1,
                      "monitor_timer": 10 ** 8, "ntime_visual": 10 ** 8, "ntime_animation": 10 ** 8,
                      "computation_time_timer": 10 ** 8, "block_Threads_X": 128, "block_Threads_Y": 1,
                      "block_Threads_Z": 1})
    return case


def run(precision: str = "f32", steps: int = 1000, size: int = 256, display: int = 100, workdir=None,
        timeout: float = 900.0) -> dict:
    """Run the reference program on the drainage workload; MLUPS from its own prints."""
    sys.path.insert(0, str(REPO / "mf-lbm-cuda_gb300"))
    from mflbm import cases
    exe = build(precision)
    case = drainage_case(size, steps, display)
    tmp = Path(workdir) if workdir else Path(tempfile.mkdtemp(prefix="mflbm_refcuda_"))
    try:
        cases.write_case_dir(case, str(tmp))
        t0 = time.perf_counter()
        r = subprocess.run([str(exe)], cwd=tmp, capture_output=True, text=True, timeout=timeout)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(f"reference program exited {r.returncode}:\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")
        speeds = [float(x) for x in re.findall(r"simulation speed:\s*([0-9.eE+-]+)\s*MLUPS", r.stdout)]
        total = re.findall(r"Code speed:\s*([0-9.eE+-]+)\s*MLUPS", r.stdout)
        steady = speeds[1:] if len(speeds) > 1 else speeds
        return {"precision": precision, "lattice": [size] * 3, "steps": steps, "display_every": display,
                "mlups_display": speeds, "mlups": statistics.median(steady) if steady else None,
                "mlups_total": float(total[-1]) if total else None, "wall_s": round(wall, 2),
                "block": [128, 1, 1]}
    finally:
        if workdir is None:
            shutil.rmtree(tmp, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["prepare", "build", "run"])
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--display", type=int, default=100)
    a = ap.parse_args()
    if a.what == "prepare":
        print("\n".join(map(str, prepare())))
    elif a.what == "build":
        print(build(a.precision, force=True))
    else:
        print(json.dumps(run(a.precision, a.steps, a.size, a.display)))


if __name__ == "__main__":
    main()
