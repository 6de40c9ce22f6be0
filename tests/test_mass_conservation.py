"""Mass conservation in closed domains, solid-node slots included.

The collision and the Rothman-Keller recolouring conserve each node's mass,
streaming moves populations, and the implicit bounce-back of the reference
(populations parked in solid-node slots and stale fluid-node slots) moves
them back: in a closed domain (walls and periodic axes, no inlet or outlet)
the total of the live populations (oracle_harness.live_mass) is constant up
to rounding.  The per-step relative drift must stay below one unit of
roundoff of the working precision (2^-52 in FP64, 2^-23 in FP32), summed over
the steps taken.

The reference's own monitor sums mass only over fluid nodes
(src/Monitor.cpp:34-80); the populations in flight in solid-node slots make
that sum fluctuate, so it is not the conserved quantity.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

GOLDEN = Path(__file__).resolve().parent / "golden"
CLOSED = ["closed_contact", "periodic_drop"]
EPS = {abi.MFLBM_FP64: 2.0 ** -52, abi.MFLBM_FP32: 2.0 ** -23}


def _mass(case, pdf, walls):
    k = case.control_keys()
    return H.live_mass(pdf, walls, case.shape, int(k["jper"]), int(k["kper"]))


@pytest.mark.parametrize("kind", CLOSED)
def test_oracle_conserves_mass(kind):
    """The CPU oracle (bit-identical to the reference's kernels) over 400
    steps in FP64: pins the accounting of live populations."""
    case = cases.small_case(kind)
    o = H.OracleState(case, abi.MFLBM_FP64, geometry=read_dat(GOLDEN / f"{case.name}.dat"))
    o.run(2)
    m0 = _mass(case, o.a["pdf"], o.a["walls"])
    for _ in range(4):
        o.run(100)
        m = _mass(case, o.a["pdf"], o.a["walls"])
        assert abs(m - m0) <= (o.ntime - 3) * EPS[abi.MFLBM_FP64] * m0, (m, m0)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abi.MFLBM_STRICT, abi.MFLBM_FAST], ids=["strict", "fast"])
@pytest.mark.parametrize("prec", [abi.MFLBM_FP64, abi.MFLBM_FP32], ids=["f64", "f32"])
@pytest.mark.parametrize("kind", CLOSED)
def test_gpu_conserves_mass_2000_steps(mflbm_lib, kind, prec, mode):
    from mflbm import lib
    case = cases.small_case(kind)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, info = lib.setup_case(case, prec, mode, geometry=geo, want_host_geometry=True)
    walls = info["geometry"]["walls"]
    ctx.run(1, 2)
    m0 = _mass(case, ctx.download(names=("pdf",))["pdf"], walls)
    drift = []
    for first in range(3, 2003, 500):
        ctx.run(first, 500)
        m = _mass(case, ctx.download(names=("pdf",))["pdf"], walls)
        drift.append((m - m0) / m0)
        assert abs(m - m0) <= (first + 499 - 2) * EPS[prec] * m0, (first + 499, drift)
    print(f"{kind} {'f64' if prec == abi.MFLBM_FP64 else 'f32'} relative mass drift every 500 steps:",
          " ".join(f"{d:.2e}" for d in drift))
    ctx.close()
