"""Learned warm start, end to end: training data from the batched lattice
Boltzmann runs, training of the U-Net on the GPU, and the comparison of
warm and cold starts on held-out samples.

    python -m mflbm.warmstart --train 192 --eval 24 --n 64 --epochs 20 \
        --json out.json [--model unet.npz] [--load unet.npz]

Training samples are seeded single-phase grain packs (porosity uniform in
0.3-0.7) run to a converged permeability by ``mflbm_batch`` (FP32); the
network's inputs come from the device (``mflbm_unet_features``).  Held-out
samples may be larger than the training ones (``--n-eval``: the network is
fully convolutional).  For each held-out sample the study runs
  * the FP64 cold start (rest equilibrium; the accuracy reference),
  * the plain FP32 cold start, and the cold start with 16-bit storage,
  * the warm starts: features, network inference and equilibrium fill, with
    FP32 and with 16-bit population storage, falling back to the cold start
    when the permeability after the first check interval differs from the
    prediction by more than ``--fallback`` (relative),
  * the oracle starts: the fill from the converged FP64 field itself (the
    bound on what a surrogate can give), with the collision's equilibrium
    (as the warm start) and with the reference's a17 lattice-weight
    equilibrium.
Each start is run once with k recorded every ``--every`` steps.  Two stopping
rules are read from that record: convergence (k changes by less than
``--tol``, relative, over ``--interval`` steps) and the band (k stays within
``--band``, relative, of the FP64 cold start's converged k from that step
on: "time to a converged k within 1 % of FP64").  The wall time to each is
then measured in a run of its own without checks, start-up included.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import abi, cases, lib, unet
from .permeability import converge, permeability


def sample_cases(n_samples, n, seed, porosity=(0.3, 0.7), body_force=1e-4):
    rng = np.random.default_rng(seed)
    return [cases.permeability_sample(n, float(rng.uniform(*porosity)), seed + 1 + s, body_force=body_force)
            for s in range(n_samples)]


def walls_of(case, precision=abi.MFLBM_FP32):
    return lib.set_walls(case.control(precision), case.geometry_bytes())


def nu_g(case):
    k = case.control_keys()
    return float(k["fluid1_viscosity"]), float(k["body_force_0"])


def generate(samples, tol, interval, max_steps, log=print):
    """Converged FP32 flows of `samples` (one batch graph) as (inputs, raw
    targets, fluid mask) triples, plus the convergence records."""
    out = []
    t0 = time.perf_counter()
    keep = {}

    def grab(i, ctx):
        keep[i] = ctx

    res, sec = converge(samples, abi.MFLBM_FP32, tol=tol, interval=interval, max_steps=max_steps, batched=True,
                        on_done=grab)
    for i, c in enumerate(samples):
        nu, g = nu_g(c)
        w = walls_of(c)
        t, m = unet.flow_target(keep[i], w, nu, g)
        out.append((unet.features(w, c.shape), t, m))
        keep[i].close()
    log(f"generated {len(samples)} samples in {time.perf_counter() - t0:.1f} s (stepping {sec:.1f} s)")
    return out, res


def scales_of(data):
    """Per-output scale: RMS over fluid nodes of the training targets (u and
    v share one scale: the packs are statistically symmetric in x and y)."""
    s = np.zeros(4)
    for c in range(4):
        num = sum(float((t[..., c][m > 0] ** 2).sum()) for _, t, m in data)
        den = sum(float((m > 0).sum()) for _, _, m in data)
        s[c] = np.sqrt(num / max(den, 1.0))
    s[0] = s[1] = np.sqrt(0.5 * (s[0] ** 2 + s[1] ** 2))
    return np.where(s > 0, s, 1.0).astype(np.float32)


def run_until_converged(ctx, case, tol, interval, max_steps, nt=1, check=None):
    """Steps one context until k changes by <= tol (relative) over `interval`
    steps.  check(k_first) after the first interval may return False to stop
    early (fallback).  Returns (k, steps, ok)."""
    k_prev = None
    steps = 0
    while steps < max_steps:
        ctx.run(nt, interval)
        nt += interval
        steps += interval
        k = permeability(ctx, case)
        if k_prev is None and check is not None and not check(k):
            return k, steps, False
        if k_prev is not None and abs(k - k_prev) <= tol * abs(k):
            return k, steps, True
        k_prev = k
    return k_prev, steps, True


class WarmStarter:
    """The trained network with its output scales; one device network per
    input shape."""

    def __init__(self, params, scales):
        self.params, self.scales = params, np.asarray(scales, np.float32)
        self.nets = {}

    def net(self, shape):
        nx, ny, nz = shape
        key = (nz, ny, nx)
        if key not in self.nets:
            n = unet.UNet(nz, ny, nx)
            n.set_params(self.params)
            self.nets[key] = n
        return self.nets[key]

    def predict(self, case, walls):
        x = unet.features(walls, case.shape)
        return self.net(case.shape).forward(x)

    def close(self):
        for n in self.nets.values():
            n.close()


def cold_start(ctx, info, capture=True):
    """Rest-state start-up fields (mflbm_init_fields); with capture, two steps
    first so that the step graph is captured outside the timed region."""
    if capture:
        ctx.run(1, 2)
        ctx.sync()
    ctl, der = info["control"], info["derived"]
    ctx.init_fields(ctl.initial_fluid_distribution_option, der.interface_z0, info["W_in"])


CHECKPOINTS = (0, 10, 24, 50, 100, 200, 400, 800, 1600)


def transient(ctx, case, walls, t_ref, k_ref, nu, g):
    """k / k_ref and the relative L2 error of u_z over the fluid nodes at
    CHECKPOINTS steps (even step counts: post-even populations)."""
    fl = (np.asarray(walls).reshape(case.shape[::-1]) == 0)
    ks, errs, nt, prev = [], [], 1, 0
    for c in CHECKPOINTS:
        if c > prev:
            ctx.run(nt, c - prev)
            nt += c - prev
            prev = c
        ks.append(round(permeability(ctx, case) / k_ref, 4))
        t, _ = unet.flow_target(ctx, walls, nu, g)
        errs.append(round(float(np.linalg.norm((t[..., 2] - t_ref[..., 2])[fl]) / np.linalg.norm(t_ref[..., 2][fl])), 4))
    return {"steps": list(CHECKPOINTS), "k_over_kref": ks, "uz_rel_err": errs}


def record_run(ctx, case, tol, interval, max_steps, every, check=None, on_fallback=None):
    """Steps one context and records k every `every` steps until k changes by
    <= tol (relative) over `interval` steps (or max_steps).  check(k) after
    the first `interval` steps may return False: then on_fallback() restarts
    the context (the cold start) and the run goes on from there.  Returns the
    trajectory [(steps, k)], the step of the first check after the
    fallback (or None) and the steps to the tol criterion."""
    traj, nt, steps, fell = [], 1, 0, None
    back = interval // every
    while steps < max_steps:
        ctx.run(nt, every)
        nt += every
        steps += every
        k = permeability(ctx, case)
        traj.append((steps, k))
        if check is not None and fell is None and steps == interval and not check(k):
            on_fallback()
            fell, nt = steps, 1
            continue
        if len(traj) > back and (fell is None or steps - fell >= interval):
            k_old = traj[-1 - back][1]
            if abs(k - k_old) <= tol * abs(k):
                return traj, fell, steps
    return traj, fell, steps


def band_steps(traj, k_ref, band):
    """First recorded step from which every later k lies within `band`
    (relative) of k_ref; None if the last one does not."""
    first = None
    for s, k in traj:
        if abs(k - k_ref) <= band * abs(k_ref):
            if first is None:
                first = s
        else:
            first = None
    return first


def evaluate(ws, case, tol, interval, max_steps, fallback, storage=abi.MFLBM_STORE_F16, with_transient=False,
             band=0.01, every=50):
    """One held-out sample: the FP64 cold start (the accuracy reference, and
    the converged field of the oracle start), the FP32 cold start, the cold
    start with 16-bit storage, the warm starts (FP32 and, unless `storage` is
    native, 16-bit storage) and the oracle start (equilibrium fill from the
    converged FP64 field: the best any surrogate could give through the
    equilibrium fill).  Each start is run once with k recorded every `every`
    steps, which gives the steps to the convergence criterion (tol over
    interval) and the steps after which k stays within `band` of the FP64
    cold start's converged k; each of the two step counts is then timed in
    a run of its own without checks (start-up, features and inference of the
    warm starts included).  Optionally the transients of the cold, warm and
    oracle starts (untimed runs)."""
    nu, g = nu_g(case)
    nx, ny, nz = case.shape
    rec = {"case": case.name, "porosity_target": case.geometry.porosity, "n": [nx, ny, nz]}
    ctx, info = lib.setup_case(case, abi.MFLBM_FP64, abi.MFLBM_FAST)
    walls = info["walls_global"]
    cold_start(ctx, info)
    t0 = time.perf_counter()
    k_ref, steps, _ = run_until_converged(ctx, case, tol, interval, max_steps)
    rec["fp64_cold"] = {"k": k_ref, "steps": steps, "seconds": time.perf_counter() - t0}
    t_ref, _ = unet.flow_target(ctx, walls, nu, g)
    ctx.close()
    ws.net(case.shape)              # device network of this shape, created outside the timed regions
    names = {abi.MFLBM_STORE_NATIVE: "fp32", abi.MFLBM_STORE_F16: "f16", abi.MFLBM_STORE_BF16: "bf16"}
    variants = [("fp32_cold", abi.MFLBM_STORE_NATIVE, "cold"), ("warm_fp32", abi.MFLBM_STORE_NATIVE, "warm"),
                ("oracle_fp32", abi.MFLBM_STORE_NATIVE, "oracle"), ("oracle_a17", abi.MFLBM_STORE_NATIVE, "oracle_a17")]
    if storage != abi.MFLBM_STORE_NATIVE:
        variants += [("cold", storage, "cold"), ("warm", storage, "warm")]
    k_pred = None

    def start(ctx, info, how):
        nonlocal k_pred
        if how == "warm":
            y = ws.predict(case, walls)
            k_pred = unet.predicted_permeability(y, ws.scales, nx, ny, nz, walls)
            unet.fill_from_prediction(ctx, y, walls, nu, g, ws.scales)
        elif how == "oracle":
            unet.fill_from_prediction(ctx, t_ref / ws.scales, walls, nu, g, ws.scales)
        elif how == "oracle_a17":
            unet.fill_from_prediction(ctx, t_ref / ws.scales, walls, nu, g, ws.scales, mrt=False)

    def timed(st, how, n_steps, fell):
        """Wall seconds of the start plus n_steps steps (the fallback, if the
        recorded run took it, at the same step), no checks in between."""
        ctx, info = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, storage=st)
        cold_start(ctx, info)
        ctx.sync()
        t0 = time.perf_counter()
        start(ctx, info, how)
        if fell is not None and n_steps > fell:
            ctx.run(1, fell)
            permeability(ctx, case)
            cold_start(ctx, info, capture=False)
            ctx.run(1, n_steps - fell)
        else:
            ctx.run(1, n_steps)
        ctx.sync()
        sec = time.perf_counter() - t0
        ctx.close()
        return sec

    for name, st, how in variants:
        ctx, info = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, storage=st)
        cold_start(ctx, info)
        t0 = time.perf_counter()
        start(ctx, info, how)
        t_start = time.perf_counter() - t0
        check = None
        if how == "warm":
            kp = k_pred
            check = lambda k1: abs(k1 - kp) <= fallback * abs(k1)
        traj, fell, steps = record_run(ctx, case, tol, interval, max_steps, every, check,
                                       on_fallback=lambda: cold_start(ctx, info, capture=False))
        ctx.close()
        k = traj[-1][1]
        nb = band_steps(traj, k_ref, band)
        r = {"k": k, "steps": steps, "seconds": timed(st, how, steps, fell), "start_seconds": t_start,
             "fallback": fell is not None, "storage": names[st], "k_rel_err": abs(k - k_ref) / abs(k_ref),
             "band_steps": nb, "band_seconds": timed(st, how, nb, fell) if nb else None,
             "k_traj": [round(kk / k_ref, 5) for _, kk in traj[:40]]}
        rec[name] = r
        if with_transient and st == abi.MFLBM_STORE_NATIVE:
            ctx, info = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST)
            start(ctx, info, how)
            rec[name]["transient"] = transient(ctx, case, walls, t_ref, k_ref, nu, g)
            ctx.close()
    rec["k_predicted"] = k_pred
    rec["k_pred_rel_err"] = abs(k_pred - k_ref) / abs(k_ref)
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=192)
    ap.add_argument("--eval", type=int, default=24)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--n-eval", type=int, default=0, help="lattice size of the held-out samples (default --n)")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--interval", type=int, default=500)
    ap.add_argument("--max-steps", type=int, default=100000)
    ap.add_argument("--fallback", type=float, default=0.5)
    ap.add_argument("--storage", default="f16", choices=["native", "f16", "bf16"])
    ap.add_argument("--seed", type=int, default=20000)
    ap.add_argument("--model", default="", help="write the trained parameters here (.npz)")
    ap.add_argument("--load", default="", help="skip data generation and training: use these parameters")
    ap.add_argument("--transient", type=int, default=0, help="record the transients of the first N held-out samples")
    ap.add_argument("--band", type=float, default=0.01, help="k within this of the FP64 cold start's (relative)")
    ap.add_argument("--every", type=int, default=50, help="steps between recorded k")
    ap.add_argument("--json", default="")
    a = ap.parse_args()
    st = {"native": abi.MFLBM_STORE_NATIVE, "f16": abi.MFLBM_STORE_F16, "bf16": abi.MFLBM_STORE_BF16}[a.storage]
    out = {"config": vars(a)}
    log = lambda s: print(s, flush=True)
    if a.load:
        params, scales = unet.load_model(a.load)
    else:
        train_cases = sample_cases(a.train, a.n, a.seed)
        data, res = generate(train_cases, a.tol, a.interval, a.max_steps, log)
        out["train_steps"] = [r["steps"] for r in res]
        scales = scales_of(data)
        norm = [(x, t / scales, m) for x, t, m in data]
        net = unet.UNet(a.n, a.n, a.n, seed=a.seed)
        losses, sec = unet.train(net, norm, a.epochs, lr=a.lr, log=log)
        params = net.get_params()
        net.close()
        out["training"] = {"losses": losses, "seconds": sec, "samples": a.train, "epochs": a.epochs,
                           "step_ms": 1e3 * sec / (a.epochs * a.train), "scales": scales.tolist()}
        if a.model:
            unet.save(a.model, params, scales)
    ws = WarmStarter(params, scales)
    recs = []
    for i, c in enumerate(sample_cases(a.eval, a.n_eval or a.n, a.seed + 100000)):
        r = evaluate(ws, c, a.tol, a.interval, a.max_steps, a.fallback, st, with_transient=i < a.transient,
                     band=a.band, every=a.every)
        log(json.dumps(r))
        recs.append(r)
    ws.close()
    tot = lambda key, f: float(sum(r[key][f] for r in recs))
    out["samples"] = recs
    summ = {"samples": len(recs), "band": a.band, "fp64_cold_seconds": tot("fp64_cold", "seconds"),
            "fp32_cold_seconds": tot("fp32_cold", "seconds"), "fp32_cold_steps": tot("fp32_cold", "steps"),
            "max_k_rel_err_fp32_cold": max(r["fp32_cold"]["k_rel_err"] for r in recs),
            "median_k_pred_rel_err": float(np.median([r["k_pred_rel_err"] for r in recs]))}
    in_band = all(r["fp32_cold"]["band_steps"] for r in recs)
    if in_band:
        summ["fp32_cold_band_seconds"] = tot("fp32_cold", "band_seconds")
        summ["fp32_cold_band_steps"] = tot("fp32_cold", "band_steps")
    for v in [k for k in ("warm_fp32", "oracle_fp32", "oracle_a17", "cold", "warm") if k in recs[0]]:
        summ[v] = {"seconds": tot(v, "seconds"), "steps": tot(v, "steps"),
                   "speedup_vs_fp32_cold": tot("fp32_cold", "seconds") / max(tot(v, "seconds"), 1e-12),
                   "max_k_rel_err": max(r[v]["k_rel_err"] for r in recs),
                   "fallbacks": sum(r[v]["fallback"] for r in recs), "storage": recs[0][v]["storage"]}
        if in_band and all(r[v]["band_steps"] for r in recs):
            summ[v].update({"band_seconds": tot(v, "band_seconds"), "band_steps": tot(v, "band_steps"),
                            "band_speedup_vs_fp32_cold": tot("fp32_cold", "band_seconds") / tot(v, "band_seconds")})
    out["summary"] = summ
    log(json.dumps(out["summary"]))
    if a.json:
        with open(a.json, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
