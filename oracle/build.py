"""Build recipes for the CPU oracle (test infrastructure only).

``build_oracle()`` compiles the CPU restatement ``mflbm_oracle.cpp`` into
``oracle/_build/libmflbm_oracle.so``.

``build_ref()`` compiles the reference's own sources, where they lie under the
reference checkout, into ``oracle/_ref/libmflbm_ref_{f32,f64}.so``: the kernel
bodies of ``src/main_iteration_GPU.cu`` (lines 1-1888, everything before the
launch function, fed to g++ on standard input so no copy is written) as host
C++ through ``refshim/host_cuda_shim.h``, the reference's host set-up files
unchanged, a translation unit that defines the reference's globals from its
own headers, and ``refshim/ref_driver.cpp`` (the launch sequence).  Outputs go
only to ``oracle/_ref/``.  Both libraries use ``-ffp-contract=off`` so their
arithmetic is the IEEE sequence written in the sources on every host.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
# The reference checkout: $MFLBM_REFERENCE, else a "reference" folder beside
# this repository's folder.  Absent (as on a machine without the checkout),
# the reference-side recipes and tests are skipped.
REFERENCE = Path(os.environ.get("MFLBM_REFERENCE", str(REPO.parent / "reference")))
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"

FLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17"]
REF_HOST_SOURCES = ["IO_multiphase.cpp", "Init_multiphase.cpp", "Misc.cpp", "Monitor.cpp",
                    "Phase_gradient.cpp", "Geometry_preprocessing.cpp", "utils.cpp"]
KERNEL_LAST_LINE = 1888  # src/main_iteration_GPU.cu: the launch function starts at 1890


def _run(cmd, stdin=None):
    r = subprocess.run(cmd, input=stdin, capture_output=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stderr.decode(errors='replace')}")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def oracle_path() -> Path:
    return HERE / "_build" / "libmflbm_oracle.so"


def build_oracle(force: bool = False) -> Path:
    out = oracle_path()
    src = HERE / "mflbm_oracle.cpp"
    hdr = REPO / "include" / "mflbm.h"
    if force or _stale(out, [src, hdr, Path(__file__)]):
        out.parent.mkdir(parents=True, exist_ok=True)
        tmp = out.with_suffix(".so.tmp")
        _run(["g++", *FLAGS, "-shared", "-I", str(REPO / "include"), str(src), "-o", str(tmp)])
        os.replace(tmp, out)
    return out


def ref_available() -> bool:
    return (REFERENCE / "src" / "main_iteration_GPU.cu").exists()


def ref_path(precision: str) -> Path:
    return HERE / "_ref" / f"libmflbm_ref_{precision}.so"


def build_ref(force: bool = False):
    """Build oracle/_ref/libmflbm_ref_{f32,f64}.so; returns {} without a reference checkout."""
    if not ref_available():
        return {}
    outdir = HERE / "_ref"
    outdir.mkdir(parents=True, exist_ok=True)
    shim = HERE / "refshim" / "host_cuda_shim.h"
    deps = [shim, HERE / "refshim" / "ref_driver.cpp", HERE / "refshim" / "ref_globals.cpp", Path(__file__)]
    results = {}
    for prec in ("f32", "f64"):
        out = ref_path(prec)
        if not force and not _stale(out, deps):
            results[prec] = out
            continue
        inc = ["-include", str(shim), "-I", str(REFERENCE / "includes"), "-I", str(CUDA_INC), "-w"]
        if prec == "f64":
            inc = ["-DREF_DOUBLE", *inc]
        objs = []
        jobs = []
        kern_o = outdir / f"kernels_{prec}.o"
        body = subprocess.run(["sed", "-n", f"1,{KERNEL_LAST_LINE}p",
                               str(REFERENCE / "src" / "main_iteration_GPU.cu")],
                              capture_output=True, check=True).stdout
        jobs.append((["g++", *FLAGS, *inc, "-x", "c++", "-", "-c", "-o", str(kern_o)], body))
        objs.append(kern_o)
        for s in REF_HOST_SOURCES:
            o = outdir / f"{Path(s).stem}_{prec}.o"
            jobs.append((["g++", *FLAGS, *inc, "-c", str(REFERENCE / "src" / s), "-o", str(o)], None))
            objs.append(o)
        for s in ("ref_globals.cpp", "ref_driver.cpp"):
            o = outdir / f"{Path(s).stem}_{prec}.o"
            jobs.append((["g++", *FLAGS, *inc, "-c", str(HERE / "refshim" / s), "-o", str(o)], None))
            objs.append(o)
        with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
            list(ex.map(lambda j: _run(j[0], j[1]), jobs))
        tmp = out.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-fopenmp", *map(str, objs), "-o", str(tmp)])
        os.replace(tmp, out)
        results[prec] = out
    return results


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
