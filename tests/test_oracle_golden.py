"""The CPU oracle against the golden fixtures produced by the reference's own
code (tests/golden/make_golden.py): bit-exact digests of geometry, derived
parameters and every state array after 0, 1, 2, 11 and 20 steps, for six
cases that exercise every boundary kernel, in FP32 and FP64."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

GOLDEN = Path(__file__).resolve().parent / "golden"


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_oracle_matches_reference_golden(kind, prec):
    case = cases.small_case(kind)
    gold = json.loads((GOLDEN / f"{case.name}_{H.suffix(prec)}.json").read_text())
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    assert digest(geo) == gold["geometry_dat_sha256"]
    o = H.OracleState(case, prec, geometry=geo)
    for n, d in gold["geometry"].items():
        assert digest(o.a[n]) == d, f"geometry array {n} differs"
    sc = gold["scalars"]
    for n in ("lbm_gamma", "force_z", "la_nui1", "la_nui2", "lbm_beta", "phi_inlet", "sa_inject", "uin_avg",
              "relaxation", "cos_theta", "rho_in", "rho_out"):
        assert getattr(o.params, n) == sc[n], n
    for n in ("num_solid_boundary_global", "num_fluid_boundary_global", "num_solid_boundary",
              "num_fluid_boundary", "pore_sum"):
        assert getattr(o.counts, n) == sc[n], n
    done = 0
    for cp in gold["checkpoints"]:
        o.run(cp - done)
        done = cp
        for n, d in gold["state"][str(cp)].items():
            assert digest(o.a[n]) == d, f"{n} differs after {cp} steps"


def test_golden_geometry_regenerates():
    """The seeded generator still produces the committed geometry bodies."""
    for kind in cases.SMALL_KINDS:
        c = cases.small_case(kind)
        assert np.array_equal(c.geometry_bytes(), read_dat(GOLDEN / f"{c.name}.dat")), kind
