"""Errors of the reduced-precision paths against the FP64 path over a long
drainage run (the precision study): FP32 populations, and FP16 / BF16
shifted-deviation storage with FP32 collision, each stepped beside the FP64
run on the same geometry; every `interval` steps the saturation, the flow
rate (flux1 + flux2 of the FP64 monitor sums), the total mass and the RMS
difference of phi over the fluid nodes are compared with the FP64 run.

    python -m mflbm.precision [--size 384 384 512] [--steps 20000] [--interval 1000]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import abi, cases, lib

VARIANTS = (("fp32", abi.MFLBM_FP32, abi.MFLBM_STORE_NATIVE), ("f16", abi.MFLBM_FP32, abi.MFLBM_STORE_F16),
            ("bf16", abi.MFLBM_FP32, abi.MFLBM_STORE_BF16))


def study(case, steps, interval, log=print):
    geo = case.geometry_bytes()
    k = case.control_keys()
    ne_in, ne_out = int(k["n_exclude_inlet"]), int(k["n_exclude_outlet"])
    nx, ny, nz = case.shape
    ref, info = lib.setup_case(case, abi.MFLBM_FP64, abi.MFLBM_FAST, geometry=geo, want_host_geometry=True)
    walls = info["geometry"]["walls"].reshape(nz + 4, ny + 4, nx + 4)[2:nz + 2, 2:ny + 2, 2:nx + 2]
    fluid = walls == 0
    ctxs = {name: lib.setup_case(case, prec, abi.MFLBM_FAST, geometry=geo, storage=st)[0]
            for name, prec, st in VARIANTS}

    def phi(c):
        return c.download(["phi"])["phi"].reshape(nz + 8, ny + 8, nx + 8)[4:nz + 4, 4:ny + 4, 4:nx + 4][fluid]

    rows = []
    nt = 1
    seconds = {name: 0.0 for name in ["fp64"] + list(ctxs)}
    while nt <= steps:
        for name, c in [("fp64", ref)] + list(ctxs.items()):
            t0 = time.perf_counter()
            c.run(nt, interval)
            c.sync()
            seconds[name] += time.perf_counter() - t0
        nt += interval
        m0 = ref.monitor(ne_in, ne_out)
        p0 = phi(ref).astype(np.float64)
        row = {"step": nt - 1, "fp64": {"saturation": m0["saturation"], "flow_rate": m0["flux1_sum"] + m0["flux2_sum"],
                                        "total_mass": m0["total_mass"]}}
        for name, c in ctxs.items():
            m = c.monitor(ne_in, ne_out)
            fr, fr0 = m["flux1_sum"] + m["flux2_sum"], row["fp64"]["flow_rate"]
            row[name] = {"saturation_rel_err": abs(m["saturation"] - m0["saturation"]) / abs(m0["saturation"]),
                         "flow_rate_rel_err": abs(fr - fr0) / max(abs(fr0), 1e-300),
                         "total_mass_rel_err": abs(m["total_mass"] - m0["total_mass"]) / abs(m0["total_mass"]),
                         "phi_rms_err": float(np.sqrt(np.mean((phi(c).astype(np.float64) - p0) ** 2)))}
        rows.append(row)
        log(json.dumps(row))
    nodes = nx * ny * nz
    mlups = {name: nodes * (nt - 1) / s / 1e6 for name, s in seconds.items()}
    for c in [ref] + list(ctxs.values()):
        c.close()
    return rows, mlups


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, nargs=3, default=[384, 384, 512])
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--interval", type=int, default=1000)
    ap.add_argument("--json", default="")
    a = ap.parse_args()
    case = cases.precision_case(tuple(a.size))
    rows, mlups = study(case, a.steps, a.interval, log=lambda s: print(s, flush=True))
    out = {"case": case.name, "steps": a.steps, "interval": a.interval, "rows": rows, "mlups": mlups,
           "max": {name: {key: max(r[name][key] for r in rows) for key in rows[0][name]} for name in ("fp32", "f16", "bf16")}}
    print(json.dumps({"mlups": mlups, "max": out["max"]}))
    if a.json:
        with open(a.json, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
