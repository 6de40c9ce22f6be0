"""Throughput benchmark of the MF-LBM hot path on GB300.

Workload: two-phase drainage on a 256 x 256 x 256 lattice (flow along z,
walls on x and y), seeded overlapping-sphere pack r ~ U[4, 10] at porosity
0.45, tau 0.8/0.8, gamma 0.005, contact angle 30 deg, velocity inlet
u = 5e-5, convective outlet; FP32 populations (the reference's default
precision).  A step is one lattice-Boltzmann time step (collision+streaming,
boundaries, colour gradient).  MLUPS counts all lattice nodes, solids
included, as the reference does (src/main.cpp:194-197).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs under torchrun as independent replicas (one lattice per GPU, no
collective on the data path; the reference has no domain decomposition).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
PKG = REPO / "mf-lbm-cuda_gb300"
for p in (str(PKG), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)

# Algorithmic bytes per fluid-node update (FP32 populations): 38 populations
# read and written once (304 B); the phase field written by the collision and
# read by the gradient step (8 B); plus one mask byte per lattice node.
POP_BYTES = 4
STEP_BYTES_PER_FLUID = 2 * 38 * POP_BYTES + 2 * 4
# the collision kernel's share: populations in and out plus its phase-field write
COLLIDE_BYTES_PER_FLUID = 2 * 38 * POP_BYTES + 4
MASK_BYTES_PER_NODE = 1


def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [x.strip() for x in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def read_traffic_profile():
    """DRAM bytes per fluid node of the collision kernel from the committed ncu summary."""
    f = REPO / "profiles" / "collide_stream_drainage.md"
    if not f.exists():
        return None, None
    m = re.search(r"dram_bytes_per_fluid_node:\s*([0-9.]+)", f.read_text())
    return (float(m.group(1)), f.name) if m else (None, None)


def dist_setup(gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def max_over_ranks(dist, value):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def replica_mlups(world, nodes, steps, t_max_ms):
    """Whole-job MLUPS of `world` independent replicas of `nodes` lattice nodes
    each, `steps` steps, the slowest rank taking `t_max_ms`."""
    return world * nodes * steps / (t_max_ms * 1e-3) / 1e6


def cpu_reference_run(case, steps, warmup, budget_s=90.0):
    """The oracle (CPU restatement of the reference's kernels, OpenMP) on the
    same workload; the number of timed steps is capped to stay within budget."""
    sys.path.insert(0, str(REPO / "tests"))
    import oracle_harness as H
    from mflbm import abi
    geo = case.geometry_bytes()
    t0 = time.perf_counter()
    o = H.OracleState(case, abi.MFLBM_FP32, geometry=geo)
    setup_s = time.perf_counter() - t0
    threads = int(H.oracle_lib().orc_max_threads())
    t0 = time.perf_counter()
    o.run(max(1, warmup))
    t_step = (time.perf_counter() - t0) / max(1, warmup)
    n = int(max(2, min(steps, budget_s / max(t_step, 1e-6))))
    t0 = time.perf_counter()
    o.run(n)
    dt = time.perf_counter() - t0
    nx, ny, nz = case.shape
    return {"mlups": nx * ny * nz * n / dt / 1e6, "steps": n, "seconds": dt, "threads": threads,
            "setup_s": setup_s}


def _timed_run(run, sync, stream):
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    run()
    ev1.record(stream)
    sync()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def storage_variants(case, geo, steps, nt):
    """The same workload with 16-bit population storage (FP32 collision):
    MLUPS, collision time and its algorithmic bandwidth (152 + 4 B per fluid
    node for the populations and phi, + 1 B per node)."""
    import torch
    from mflbm import abi, lib
    out = {}
    nx, ny, nz = case.shape
    for name, st in (("f16", abi.MFLBM_STORE_F16), ("bf16", abi.MFLBM_STORE_BF16)):
        c, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, geometry=geo, storage=st)
        n_fluid, n_all = c.node_counts()
        c.run(1, 20)
        stream = torch.cuda.ExternalStream(c.stream())
        ms = _timed_run(lambda: c.run(21, steps), c.sync, stream)
        c.set_timing(True)
        c.run(21 + steps, 40)
        tc, tg, n = c.kernel_times()
        c.set_timing(False)
        coll = tc / max(n, 1)
        out[name] = {"value": round(n_all * steps / (ms * 1e-3) / 1e6, 2), "unit": "MLUPS",
                     "ms_per_step": round(ms / steps, 5), "collide_ms": round(coll, 5),
                     "gradient_ms": round(tg / max(n, 1), 5),
                     "collide_gbs": round((n_fluid * 156 + n_all) / (coll * 1e-3) / 1e9, 1)}
        c.close()
    return out


def fp64_variant(case, geo, steps):
    """The same workload in FP64 (populations and collision): MLUPS and the
    collision kernel's algorithmic bandwidth (616 B per fluid node + 1 B per
    node).  On GB300 the FP64 collision is bound by the FP64 pipe, not by HBM."""
    import torch
    from mflbm import abi, lib
    c, _ = lib.setup_case(case, abi.MFLBM_FP64, abi.MFLBM_FAST, geometry=geo)
    n_fluid, n_all = c.node_counts()
    c.run(1, 4)
    stream = torch.cuda.ExternalStream(c.stream())
    ms = _timed_run(lambda: c.run(5, steps), c.sync, stream)
    c.set_timing(True)
    c.run(5 + steps, 4)
    tc, tg, n = c.kernel_times()
    c.set_timing(False)
    coll = tc / max(n, 1)
    c.close()
    return {"value": round(n_all * steps / (ms * 1e-3) / 1e6, 2), "unit": "MLUPS", "ms_per_step": round(ms / steps, 5),
            "collide_ms": round(coll, 5), "gradient_ms": round(tg / max(n, 1), 5),
            "collide_gbs": round((n_fluid * 616 + n_all) / (coll * 1e-3) / 1e9, 1)}


def late_state(ctx, nt, n_all, n_fluid, target=10001, timed=200):
    """The same drainage ~10,000 steps in (the front well inside the pack):
    MLUPS over `timed` steps and the sizes of the sparse gradient sets."""
    import torch
    if nt < target:
        ctx.run(nt, target - nt)
        nt = target
    stream = torch.cuda.ExternalStream(ctx.stream())
    ms = _timed_run(lambda: ctx.run(nt, timed), ctx.sync, stream)
    nt += timed
    st = ctx.interface_stats()
    return nt, {"value": round(n_all * timed / (ms * 1e-3) / 1e6, 2), "unit": "MLUPS", "after_steps": nt - 1,
                "ms_per_step": round(ms / timed, 5), "gradient_sets": st, "super_blocks": ctx.super_block_stats(),
                "interface_fraction": round(st["interface_nodes"] / n_fluid, 5)}


def interface_rich(case, geo, timed=200, settle=20, seed=1206):
    """The worst case of the sparse colour-gradient passes: the same 256^3
    pack with phi = +-1 drawn at random per node (the reference's random
    initial distribution, initial_fluid_distribution_option 6, at saturation
    0.5; the reference draws from rand() seeded by the clock, this uses a
    seeded generator), the rest state at that phi, uploaded through the C
    ABI; MLUPS over `timed` steps after `settle` steps."""
    import torch
    from mflbm import abi, lib
    c, info = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, geometry=geo)
    nx, ny, nz = case.shape
    L = c.L
    phi = c.download(names=("phi",))["phi"].reshape(nz + 8, ny + 8, nx + 8)
    rng = np.random.default_rng(seed)
    core = phi[3:nz + 5, 3:ny + 5, 3:nx + 5]                    # nodes [0, n+1]^3
    core[...] = np.where(rng.random(core.shape) < 0.5, 1.0, -1.0).astype(np.float32)
    phi[:4, :, :] = np.float32(info["params"].phi_inlet)         # inlet ghosts k <= 0
    p1 = phi[3:nz + 5, 3:ny + 5, 3:nx + 5]                      # s1 nodes
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
    pdf = np.empty((2, 19) + p1.shape, dtype=np.float32)
    for g, sgn in ((0, 1.0), (1, -1.0)):
        r = (np.float32(1.0) + np.float32(sgn) * p1) * np.float32(0.5)
        for q in range(19):
            np.multiply(r, w[q], out=pdf[g, q])
    f_cv = np.ascontiguousarray(pdf[0, :, nz, :, :])
    g_cv = np.ascontiguousarray(pdf[1, :, nz, :, :])
    phi_cv = np.ascontiguousarray(p1[nz, :, :])                # convective outlet state: z = nz
    c.upload_fields(pdf=pdf.reshape(-1), phi=phi.reshape(-1), W_in=info["W_in"], f_convec_bc=f_cv.reshape(-1),
                    g_convec_bc=g_cv.reshape(-1), phi_convec_bc=phi_cv.reshape(-1))
    del pdf
    n_fluid, n_all = c.node_counts()
    c.run(1, settle)
    stream = torch.cuda.ExternalStream(c.stream())
    ms = _timed_run(lambda: c.run(1 + settle, timed), c.sync, stream)
    st = c.interface_stats()
    sb = c.super_block_stats()
    c.close()
    return {"value": round(n_all * timed / (ms * 1e-3) / 1e6, 2), "unit": "MLUPS", "ms_per_step": round(ms / timed, 5),
            "after_steps": settle + timed, "gradient_sets": st, "super_blocks": sb,
            "interface_fraction": round(st["interface_nodes"] / n_fluid, 5),
            "how": "random phi = +-1 per node (seeded), rest state, uploaded through mflbm_upload_fields"}


def reference_cuda(size):
    """The reference's own CUDA program (baseline/ref_cuda.py: its kernels and
    host program compiled for sm_103a with two documented allocation/print
    patches) on the same workload: MLUPS from its own prints, FP32 and FP64."""
    sys.path.insert(0, str(REPO / "baseline"))
    import ref_cuda
    if not ref_cuda.available("f32"):
        return {"unavailable": "patched reference sources not present (baseline/ref_cuda.py prepare, "
                               "on a machine with the reference checkout)"}
    out = {}
    for prec, steps, disp in (("f32", 600, 100), ("f64", 200, 50)):
        try:
            r = ref_cuda.run(prec, steps=steps, size=size, display=disp)
            out[prec] = {"value": round(r["mlups"], 2) if r["mlups"] else None, "unit": "MLUPS",
                         "steps": steps, "mlups_display": r["mlups_display"], "mlups_total": r["mlups_total"],
                         "block": r["block"]}
        except Exception as e:   # keep the bench line whatever happens here
            out[prec] = {"error": str(e)[-400:]}
    out["patches"] = [p[3] for p in ref_cuda.PATCHES]
    out["how"] = ("median of the program's own 'simulation speed' prints (all nodes x steps / wall time "
                  "between prints, src/main.cpp:191-199), block 128x1x1 from the control file")
    return out


def batch_vs_sequential(steps):
    """16 single-phase samples of 48^3 .. 96^3 (porosity 0.3 .. 0.7) stepped
    together by mflbm_batch_run (persistent launches with grid barriers, block
    size and tile shape from mflbm_batch_autotune) against each context's own
    graph replays, one context after another (each context autotuned alone)."""
    from mflbm import abi, lib, permeability
    samples = permeability.make_samples(16, 48, 96)
    ctxs = [lib.setup_case(s, abi.MFLBM_FP32, abi.MFLBM_FAST)[0] for s in samples]
    solo = [lib.setup_case(s, abi.MFLBM_FP32, abi.MFLBM_FAST)[0] for s in samples]
    nodes = sum(int(np.prod(s.shape)) for s in samples)
    steps += steps & 1
    b = lib.Batch(ctxs)
    b.run(1, 4)
    tuned = b.autotune(2)
    for c in solo:
        c.run(1, 4)
        c.autotune(2)
    b.run(5, 4)
    for c in solo:
        c.run(5, 4)
        c.sync()
    t0 = time.perf_counter()
    b.run(9, steps)
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    for c in solo:
        c.run(9, steps)
    for c in solo:
        c.sync()
    t_seq = time.perf_counter() - t0
    opts = b.options()
    same = all(np.array_equal(x.download(names=("pdf",))["pdf"], y.download(names=("pdf",))["pdf"])
               for x, y in zip(ctxs, solo))
    b.close()
    for c in ctxs + solo:
        c.close()
    return {"samples": len(samples), "sizes": [s.shape[0] for s in samples], "steps": steps,
            "batched_mlups": round(nodes * steps / t_batch / 1e6, 1),
            "sequential_mlups": round(nodes * steps / t_seq / 1e6, 1),
            "batched_over_sequential": round(t_seq / t_batch, 3),
            "mode": {1: "graph", 2: "persistent"}.get(opts["used_mode"], "?"), "grid": opts["grid"],
            "block": opts["block"], "tile_bricks": [tuned["tile_x"], tuned["tile_y"], tuned["tile_z"]],
            "results_identical": bool(same),
            "how": "wall clock, mflbm_batch_run (one persistent launch per 100 steps) vs mflbm_run per context "
                   "(graph replays), FP32 fast, same start states"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=256, help="lattice edge (default: the 256^3 workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the 16-bit storage and batch measurements")
    ap.add_argument("--no-tune", action="store_true", help="keep the default block sizes (no autotuning)")
    ap.add_argument("--storage", default="native", choices=["native", "f16", "bf16"],
                    help="population storage of the main run (default: FP32 populations; f16 / bf16 for "
                         "one-kernel captures of the 16-bit collision)")
    ap.add_argument("--interface-rich-only", action="store_true",
                    help="run only the interface-rich state (random +-1 phi) for --warmup + --steps steps and "
                         "print its line (for launch lists of the sparse passes' worst case)")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip the reference's own CUDA program (built from baseline/_ref when present)")
    args = ap.parse_args()
    warmup = max(3, args.warmup)

    from mflbm import abi, cases
    case = cases.drainage_256x256x256()
    if args.size != 256:
        case.keys.update({"nxGlobal": args.size, "nyGlobal": args.size, "nzGlobal": args.size})
        case.name = f"drainage_{args.size}x{args.size}x{args.size}"
    nx, ny, nz = case.shape
    n_all = nx * ny * nz
    metric = f"MLUPS at {nx}^3 (all-node lattice updates per second, reference definition)"
    data = ("synthetic: seeded overlapping-sphere pack, radii U[4,10], porosity 0.45, seed 1200, "
            "2-layer inlet/outlet buffers (stands in for the reference's micro-CT inputs)")

    rank, world, local, dist = dist_setup(args.gpus)

    if args.impl == "reference":
        if rank != 0:
            return
        r = cpu_reference_run(case, args.steps, warmup)
        line = {"impl": "reference", "metric": metric, "value": round(r["mlups"], 3), "unit": "MLUPS",
                "n_gpus": args.gpus, "steps": r["steps"], "warmup": warmup,
                "ms_per_step": r["seconds"] / r["steps"] * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": data,
                "config": {"workload": case.name, "lattice": [nx, ny, nz], "precision": "fp32"},
                "cpu_baseline": {"value": round(r["mlups"], 3), "unit": "MLUPS", "cores": r["threads"],
                                 "kind": "port",
                                 "sample": f"{r['steps']} time steps of the full {nx}^3 workload after {warmup} "
                                           f"warm-up steps (oracle: CPU restatement of the reference kernels, "
                                           f"OpenMP, {r['threads']} threads); reference checkout absent on this host"},
                "e2e": {"value": round(r["mlups"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    from mflbm import lib
    lib.load()
    geo = case.geometry_bytes()
    if args.interface_rich_only:
        print(json.dumps({"interface_rich": interface_rich(case, geo, timed=args.steps, settle=max(args.warmup, 2) // 2 * 2)}))
        return
    storage = {"native": abi.MFLBM_STORE_NATIVE, "f16": abi.MFLBM_STORE_F16, "bf16": abi.MFLBM_STORE_BF16}[args.storage]
    pop_bytes = POP_BYTES if storage == abi.MFLBM_STORE_NATIVE else 2
    ctx, info = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, geometry=geo, storage=storage)
    n_fluid, _ = ctx.node_counts()
    porosity = n_fluid / n_all

    # launches per step (counted on eager steps)
    c0 = lib.load().mflbm_kernel_launch_count()
    ctx.step(1)
    ctx.step(2)
    ctx.sync()
    launches_per_step = (lib.load().mflbm_kernel_launch_count() - c0) / 2
    nt = 3
    ctx.run(nt, warmup)
    nt += warmup
    ctx.sync()
    # block sizes of the step kernels from the library's autotuner (state unchanged)
    tuning = None
    if not args.no_tune:
        t = ctx.autotune(3)
        tuning = {k: t[k] for k in ("collide_block", "normals_block", "curvature_block", "extrapolate_block")}
        tuning["population_tile_bricks"] = [t["tile_x"], t["tile_y"], t["tile_z"]]

    # ---- timed region: K steps, state resident in HBM, graph-replayed ----
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(dist)
    torch.cuda.synchronize()
    ev0.record(stream)
    ctx.run(nt, args.steps)
    ev1.record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    nt += args.steps
    t_max = max_over_ranks(dist, elapsed_ms)
    value = replica_mlups(world, n_all, args.steps, t_max)

    # ---- per-kernel device time of the collision (events on the launching stream) ----
    ktime_steps = min(args.steps, 200)
    ctx.set_timing(True)
    ctx.run(nt, ktime_steps)
    nt += ktime_steps
    tc, tg, ncoll = ctx.kernel_times()
    ctx.set_timing(False)
    collide_ms = tc / max(ncoll, 1)
    gradient_ms = tg / max(ncoll, 1)
    hbm, peak_kind = peaks()
    coll_bytes = n_fluid * (2 * 38 * pop_bytes + 4) + n_all * MASK_BYTES_PER_NODE
    achieved = coll_bytes / (collide_ms * 1e-3) / 1e9
    traffic_per_fluid, traffic_src = read_traffic_profile() if storage == abi.MFLBM_STORE_NATIVE else (None, None)
    step_bytes = n_fluid * (2 * 38 * pop_bytes + 2 * 4) + n_all * MASK_BYTES_PER_NODE
    step_ms = t_max / args.steps

    # ---- end to end through the C ABI with pinned host buffers ----
    e2e_steps = min(args.steps, 200)
    L = ctx.L
    host = {}
    for n in ("pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "f_convec_bc", "g_convec_bc",
              "phi_convec_bc", "W_in"):
        shape = L.shape(abi.FIELD_KINDS[n])
        host[n] = torch.empty(int(np.prod(shape)), dtype=torch.float32, pin_memory=True).numpy().reshape(shape)
    d = ctx.download()
    for n, a in d.items():
        host[n][...] = a
    host["W_in"][...] = info["W_in"]
    h2d = sum(host[n].nbytes for n in host)
    d2h = sum(host[n].nbytes for n in host if n != "W_in")
    barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.upload_fields(**host)      # blocks until the state is on the device
    t1 = time.perf_counter()
    for s in range(e2e_steps):
        ctx.step(nt + s)
    ctx.sync()
    t2 = time.perf_counter()
    out = ctx.download(out=host)   # into the same pinned buffers
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"upload_s": round(t1 - t0, 5), "steps_s": round(t2 - t1, 5),
                 "download_s": round(time.perf_counter() - t2, 5)}
    barrier(dist)
    nt += e2e_steps
    e2e_s = max_over_ranks(dist, e2e_s)
    e2e_value = world * n_all * e2e_steps / e2e_s / 1e6
    assert np.isfinite(out["phi"]).all()

    sparse = ctx.interface_stats()
    super_blocks = ctx.super_block_stats()
    mon = ctx.monitor(2, 2)
    extra = {}
    if not args.no_extras:
        nt, extra["late_state"] = late_state(ctx, nt, n_all, n_fluid)
        ctx.close()
        extra["interface_rich"] = interface_rich(case, geo)
        extra["storage"] = storage_variants(case, geo, min(args.steps, 200), nt)
        extra["fp64"] = fp64_variant(case, geo, min(args.steps, 40))
        extra["batch"] = batch_vs_sequential(200)   # fixed: a 20-step window is mostly launch and sync noise
        if not args.no_reference_cuda and world == 1:
            extra["reference_cuda"] = reference_cuda(nx)

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        r = cpu_reference_run(case, 40, 3, budget_s=20.0)
        cpu = {"value": round(r["mlups"], 3), "unit": "MLUPS", "cores": r["threads"], "kind": "port",
               "sample": f"{r['steps']} time steps of the full {nx}^3 workload on the host cores "
                         f"(oracle: CPU restatement of the reference kernels, OpenMP, FP32)"}
    line = {
        "metric": metric, "value": round(value, 2), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": round(step_ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": data,
        "config": {"workload": case.name, "lattice": [nx, ny, nz], "fluid_nodes": n_fluid,
                   "porosity": round(porosity, 4),
                   "precision": ("fp32 populations, fp32 collision" if storage == abi.MFLBM_STORE_NATIVE
                                 else f"{args.storage} shifted populations, fp32 collision"),
                   "fp_mode": "fast", "l2": "inputs larger than L2 (populations 2.6 GB per replica), no flush",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "block_sizes": tuning or "defaults (128)"},
        "mflups": round(world * n_fluid * args.steps / (t_max * 1e-3) / 1e6, 2),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_kind": peak_kind,
                     "kernel": "collide_stream_kernel<float>", "kernel_ms": round(collide_ms, 5),
                     "algorithmic_bytes_per_launch": coll_bytes,
                     "traffic": (round(traffic_per_fluid * n_fluid) if traffic_per_fluid else None),
                     "traffic_source": traffic_src},
        "step_roofline": {"achieved": round(step_bytes / (step_ms * 1e-3) / 1e9, 1), "unit": "GB/s",
                          "frac": round(step_bytes / (step_ms * 1e-3) / 1e9 / hbm, 4),
                          "algorithmic_bytes_per_step": step_bytes, "gradient_ms": round(gradient_ms, 5)},
        "e2e": {"value": round(e2e_value, 2), "unit": "MLUPS", "steps": e2e_steps,
                "h2d_bytes_per_step": int(h2d / e2e_steps), "d2h_bytes_per_step": int(d2h / e2e_steps),
                "parts": e2e_parts, "h2d_gbs": round(h2d / e2e_parts["upload_s"] / 1e9, 1),
                "d2h_gbs": round(d2h / e2e_parts["download_s"] / 1e9, 1),
                "how": "mflbm_upload_fields from pinned host buffers, mflbm_step per step, mflbm_download_fields"},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clocks,
        "saturation": round(mon["saturation"], 6),
        # fluid nodes with a non-zero phase gradient at the end of the e2e leg: the
        # curvature gathers run only there (elsewhere the surface force is zero)
        # sizes of the last gradient pass's sparse sets (interface nodes, solid
        # nodes given a normal, fluid nodes whose normal was recomputed)
        "gradient_sets": sparse, "super_blocks": super_blocks,
        "interface_fraction": round(float(np.count_nonzero(
            out["c_norm"].reshape(nz + 4, ny + 4, nx + 4)[2:nz + 2, 2:ny + 2, 2:nx + 2])) / n_fluid, 5),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    line.update(extra)
    print(json.dumps(line))
    ctx.close()


if __name__ == "__main__":
    main()
