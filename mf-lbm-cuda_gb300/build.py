"""Build libmflbm.so (sm_103a) in-tree: mf-lbm-cuda_gb300/lib/libmflbm.so.

Translation units compile in parallel:
  step_fast.cu    step kernels with FMA contraction (production flavour)
  step_strict.cu  the same kernels with -fmad=false (IEEE ops in reference order)
  setup.cu        geometry preprocessing, start-up fields, FP64 reductions (-fmad=false)
  output.cu       VTK and checkpoint files in the reference's formats (-fmad=false)
  capi.cu         the C ABI
  unet.cu         the 3-D U-Net warm start (BF16 tensor-core convolutions and their gradients)
  host_setup.cpp  host parameter derivation and inlet profile (g++ -ffp-contract=off)
and the stand-alone program lib/mflbm_main (driver.cpp, g++, linked to the library).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
REPO = PKG.parent
LIB = OUT / "libmflbm.so"

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", *ARCH]
UNITS = {
    "step_fast.cu": [],
    "step_strict.cu": ["-fmad=false"],
    "setup.cu": ["-fmad=false"],
    "output.cu": ["-fmad=false"],
    "capi.cu": [],
    "unet.cu": [],
}
HEADERS = ["common.cuh", "context.cuh", "step_kernels.cuh", "collide.cuh", "gradient.cuh", "boundary.cuh", "setup.cuh",
           "batch.cuh", "unet_kernels.cuh", "unet_tc.cuh", "unet_halo.cuh"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    hdrs = [CSRC / h for h in HEADERS] + [REPO / "include" / "mflbm.h", Path(__file__)]
    jobs, objs = [], []
    for src, extra in UNITS.items():
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        if force or ptxas_info or _stale(obj, [CSRC / src, *hdrs]):
            flags = list(NVFLAGS) + extra + (["-Xptxas", "-v"] if ptxas_info else [])
            jobs.append([NVCC, *flags, "-c", str(CSRC / src), "-o", str(obj)])
    host_obj = OUT / "host_setup.o"
    objs.append(host_obj)
    if force or _stale(host_obj, [CSRC / "host_setup.cpp", *hdrs]):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", str(CSRC / "host_setup.cpp"),
                     "-o", str(host_obj)])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for l in logs:
            sys.stdout.write(l)
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    build_refshim(force)
    build_driver(force)
    return LIB


DRIVER = OUT / "mflbm_main"


def build_driver(force: bool = False):
    """The stand-alone program (csrc/driver.cpp) on libmflbm.so."""
    src = CSRC / "driver.cpp"
    if not force and not _stale(DRIVER, [src, REPO / "include" / "mflbm.h", LIB]):
        return DRIVER
    tmp = DRIVER.with_name(DRIVER.name + ".tmp")
    _run(["g++", "-O2", "-std=c++17", str(src), "-L", str(OUT), "-lmflbm", "-Wl,-rpath,$ORIGIN", "-o", str(tmp)])
    os.replace(tmp, DRIVER)
    return DRIVER


def refshim_path(precision: str) -> Path:
    return OUT / f"libmflbm_refshim_{precision}.a"


def build_refshim(force: bool = False):
    """Static archives with the reference's GPU entry points (include/mflbm_refshim.h)."""
    src = CSRC / "refshim.cpp"
    deps = [src, REPO / "include" / "mflbm.h", REPO / "include" / "mflbm_refshim.h"]
    for prec, define in (("f32", []), ("f64", ["-DMFLBM_REF_DOUBLE"])):
        out = refshim_path(prec)
        if not force and not _stale(out, deps):
            continue
        obj = OUT / f"refshim_{prec}.o"
        _run(["g++", "-O2", "-std=c++17", "-fPIC", *define, "-c", str(src), "-o", str(obj)])
        if out.exists():
            out.unlink()
        _run(["ar", "rcs", str(out), str(obj)])


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
