"""Live pinning of the CPU oracle against the reference compiled as host code
(oracle/_ref), where the reference checkout is available: a fresh geometry
seed per case, bit-exact after 1, 2 and 7 steps.  Skipped elsewhere (the
golden fixtures carry the same check)."""
import multiprocessing as mp

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from oracle import build as obuild

pytestmark = pytest.mark.skipif(not obuild.ref_available(), reason="reference checkout not present")

CPS = [1, 2, 7]


def _ref(args):
    kind, prec, seed = args
    import oracle_harness as HH
    from mflbm import cases as cc
    case = cc.small_case(kind, n=(16, 16, 22), seed=seed)
    return HH.run_reference_case(case, prec, CPS)


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
def test_oracle_equals_reference_all_cases(prec):
    jobs = [(k, prec, 101 + i) for i, k in enumerate(cases.SMALL_KINDS)]
    with mp.get_context("spawn").Pool(4, maxtasksperchild=1) as pool:
        refs = pool.map(_ref, jobs)
    for (kind, _, seed), ref in zip(jobs, refs):
        case = cases.small_case(kind, n=(16, 16, 22), seed=seed)
        o = H.OracleState(case, prec)
        for n, a in ref["_geometry"].items():
            assert np.array_equal(a, o.a[n]), (kind, n)
        done = 0
        for cp in CPS:
            o.run(cp - done)
            done = cp
            for n, a in ref[cp].items():
                if a is None:  # buffers the reference allocates only for its own outlet type
                    continue
                assert a.tobytes() == o.a[n].tobytes(), (kind, cp, n)
