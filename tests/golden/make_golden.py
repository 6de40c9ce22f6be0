"""Generate the golden fixtures in this folder from the reference itself.

For every small case of ``mflbm.cases.SMALL_KINDS`` and both precisions, the
reference's own kernels and set-up (compiled as host code into oracle/_ref by
oracle/build.py, from the reference checkout) run the case; the SHA-256 of
every state array at a few steps, the derived scalars, the geometry arrays
and the reference's output files after the last step (VTK types 1-3, the
geometry VTK, the checkpoint) are written to ``<case>_<f32|f64>.json``; the geometry body used is written
to ``<case>.dat``.  The CPU tests compare the oracle against these files
bit for bit.

Run from the repository root:  python tests/golden/make_golden.py
(needs the reference checkout; each case runs in a fresh process because the
reference keeps its state in globals).
"""
from __future__ import annotations

import hashlib
import json
import multiprocessing as mp
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "tests"))
sys.path.insert(0, str(REPO / "mf-lbm-cuda_gb300"))

CHECKPOINTS = [0, 1, 2, 11, 20]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _job(args):
    kind, prec = args
    import oracle_harness as H
    from mflbm import cases
    from mflbm.geometry import read_dat
    case = cases.small_case(kind)
    geo = read_dat(HERE / f"{case.name}.dat")
    out = H.run_reference_case(case, prec, CHECKPOINTS, geometry=geo, outputs=True)
    res = {"case": case.name, "kind": kind, "precision": "f32" if prec == 1 else "f64",
           "checkpoints": CHECKPOINTS, "scalars": out["_scalars"],
           "geometry": {n: digest(a) for n, a in out["_geometry"].items()},
           "state": {str(cp): {n: digest(a) for n, a in out[cp].items() if a is not None} for cp in CHECKPOINTS},
           "summary": {str(cp): {"phi_sum": float(np.sum(out[cp]["phi"].astype(np.float64))),
                                 "pdf_sum": float(np.sum(out[cp]["pdf"].astype(np.float64)))}
                       for cp in CHECKPOINTS},
           "geometry_dat_sha256": digest(geo),
           "outputs": {"step": CHECKPOINTS[-1], "sha256": out["_outputs"]}}
    return res


def main():
    from mflbm import cases
    from mflbm.geometry import write_dat
    for kind in cases.SMALL_KINDS:
        c = cases.small_case(kind)
        write_dat(HERE / f"{c.name}.dat", c.geometry_bytes())
    ctx = mp.get_context("spawn")
    jobs = [(k, p) for k in cases.SMALL_KINDS for p in (1, 2)]
    with ctx.Pool(4, maxtasksperchild=1) as pool:
        for res in pool.imap_unordered(_job, jobs):
            name = f"{res['case']}_{res['precision']}.json"
            (HERE / name).write_text(json.dumps(res, indent=1, sort_keys=True))
            print("wrote", name)


if __name__ == "__main__":
    main()
