"""Permeability of single-phase samples, run to convergence one by one or as a
batch (``mflbm_batch``: one CUDA graph launch steps every sample).

The reference has no permeability output; it is derived the way its
flowrate_time.dat allows (src/Monitor.cpp:150-193): k = nu * u_D / g, with
u_D the superficial (Darcy) velocity -- the FP64 sum of the z velocity over
the fluid nodes (``flux1_sum + flux2_sum`` of ``mflbm_monitor_reduce``) divided
by the volume inside the x walls, (nx - 2) * ny * nz -- nu the kinematic
viscosity and g the body force.  A sample has converged when k changes by
less than ``tol`` (relative) over ``interval`` steps.

    python -m mflbm.permeability --samples 8 --nmin 48 --nmax 96 [--storage f16]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import abi, cases, lib


def permeability(ctx, case):
    k = case.control_keys()
    nx, ny, nz = case.shape
    m = ctx.monitor(0, 0)
    u_d = (m["flux1_sum"] + m["flux2_sum"]) / ((nx - 2) * ny * nz)
    return float(k["fluid1_viscosity"]) * u_d / float(k["body_force_0"])


def make_samples(n_samples, nmin, nmax, seed=4000, porosity=(0.3, 0.7)):
    """Seeded cubic samples with sizes uniform in [nmin, nmax] and porosities
    uniform in `porosity` (the batching configuration's distributions)."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_samples):
        n = int(rng.integers(nmin, nmax + 1))
        out.append(cases.permeability_sample(n, float(rng.uniform(*porosity)), seed + s))
    return out


def converge(samples, precision=abi.MFLBM_FP32, fp_mode=abi.MFLBM_FAST, storage=abi.MFLBM_STORE_NATIVE,
             tol=1e-6, interval=1000, max_steps=200000, batched=True, tune=False, on_done=None):
    """Run every sample until k converges.  Returns one dict per sample
    (k, steps) and the wall time of the stepping.  on_done(i, ctx), when
    given, receives every context at the end (and then owns it); otherwise
    the contexts are closed."""
    ctxs = [lib.setup_case(c, precision, fp_mode, storage=storage)[0] for c in samples]
    if tune:
        for c in ctxs:
            c.autotune(3)
    k_prev = [None] * len(samples)
    res = [None] * len(samples)
    active = list(range(len(samples)))
    nt = 1
    t0 = time.perf_counter()
    batch, batch_set = None, None
    while active and nt <= max_steps:
        if batched:
            if batch_set != active:          # re-captured only when a sample has converged
                if batch:
                    batch.close()
                batch, batch_set = lib.Batch([ctxs[i] for i in active]), list(active)
            batch.run(nt, interval)
        else:
            for i in active:
                ctxs[i].run(nt, interval)
                ctxs[i].sync()
        nt += interval
        still = []
        for i in active:
            k = permeability(ctxs[i], samples[i])
            if k_prev[i] is not None and abs(k - k_prev[i]) <= tol * abs(k):
                res[i] = {"case": samples[i].name, "k": k, "steps": nt - 1}
            else:
                still.append(i)
            k_prev[i] = k
        active = still
    seconds = time.perf_counter() - t0
    if batch:
        batch.close()
    for i in active:
        res[i] = {"case": samples[i].name, "k": k_prev[i], "steps": nt - 1, "converged": False}
    for i, c in enumerate(ctxs):
        if on_done:
            on_done(i, c)
        else:
            c.close()
    return res, seconds


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=8)
    ap.add_argument("--nmin", type=int, default=48)
    ap.add_argument("--nmax", type=int, default=96)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--interval", type=int, default=1000)
    ap.add_argument("--max-steps", type=int, default=100000)
    ap.add_argument("--json", default="")
    ap.add_argument("--storage", default="native", choices=["native", "f16", "bf16"])
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--sequential", action="store_true")
    a = ap.parse_args()
    st = {"native": abi.MFLBM_STORE_NATIVE, "f16": abi.MFLBM_STORE_F16, "bf16": abi.MFLBM_STORE_BF16}[a.storage]
    samples = make_samples(a.samples, a.nmin, a.nmax)
    res, sec = converge(samples, abi.MFLBM_FP64 if a.fp64 else abi.MFLBM_FP32, storage=st, tol=a.tol,
                        interval=a.interval, max_steps=a.max_steps, batched=not a.sequential)
    nodes = sum(int(np.prod(s.shape)) * r["steps"] for s, r in zip(samples, res))
    out = {"mode": "sequential" if a.sequential else "batched", "samples": res, "seconds": sec,
           "lattice_updates": nodes, "aggregate_mlups": nodes / sec / 1e6,
           "converged": sum(r.get("converged", True) for r in res)}
    print(json.dumps({k: v for k, v in out.items() if k != "samples"}))
    if a.json:
        with open(a.json, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
