"""Batches and the block-size autotuner (no reference counterpart; checked
against the library's own unbatched, untuned path, strict flavour, bit for bit):

  * a batch of contexts of different sizes and boundary conditions reaches
    exactly the states each context reaches when stepped alone;
  * a context changed after the batch was captured is re-captured;
  * mflbm_autotune leaves the state unchanged and the following steps give
    the same results as with the default block sizes (each node's arithmetic
    does not depend on the launch shape);
  * a permeability sample converges, and its FP32 permeability is within 1 %
    of the FP64 one.
"""
from pathlib import Path

import pytest

from mflbm import abi, cases, permeability
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _ctx(kind, prec=abi.MFLBM_FP32, **kw):
    from mflbm import lib
    case = cases.small_case(kind)
    return lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=read_dat(GOLDEN / f"{case.name}.dat"), **kw)[0]


def _same(a, b):
    da, db = a.download(), b.download()
    return all(da[n].tobytes() == db[n].tobytes() for n in da)


def test_batch_equals_separate_runs(mflbm_lib):
    from mflbm import lib
    kinds = ["velocity_convective", "pressure_pressure", "periodic_drop"]
    solo = [_ctx(k) for k in kinds]
    grouped = [_ctx(k) for k in kinds] + [lib.setup_case(cases.permeability_sample(24, 0.5, 4100),
                                                         abi.MFLBM_FP32, abi.MFLBM_STRICT)[0]]
    alone = lib.setup_case(cases.permeability_sample(24, 0.5, 4100), abi.MFLBM_FP32, abi.MFLBM_STRICT)[0]
    b = lib.Batch(grouped)
    b.run(1, 10)
    b.run(11, 6)
    for c in solo + [alone]:
        c.run(1, 16)
    for s, g in zip(solo + [alone], grouped):
        assert _same(s, g)
    # a changed context is re-captured: new block sizes, same arithmetic
    grouped[0].set_tuning(collide=64)
    b.run(17, 4)
    for c in solo + [alone]:
        c.run(17, 4)
    for s, g in zip(solo + [alone], grouped):
        assert _same(s, g)
    b.close()
    for c in solo + grouped + [alone]:
        c.close()


@pytest.mark.parametrize("store", [abi.MFLBM_STORE_NATIVE, abi.MFLBM_STORE_F16], ids=["native", "f16"])
def test_autotune_keeps_state_and_results(mflbm_lib, store):
    a = _ctx("velocity_convective", storage=store)
    b = _ctx("velocity_convective", storage=store)
    a.run(1, 6)
    b.run(1, 6)
    t = a.autotune(2)
    for n in ("collide_block", "normals_block", "curvature_block", "extrapolate_block"):
        assert t[n] in (64, 128, 256)
    assert t["step_ms_after"] <= t["step_ms_before"] * 1.0001
    assert _same(a, b)
    a.run(7, 8)
    b.run(7, 8)
    assert _same(a, b)
    a.close()
    b.close()


def test_permeability_converges_fp32_within_1pct_of_fp64(mflbm_lib):
    samples = [cases.permeability_sample(32, 0.55, 4200)]
    r64, _ = permeability.converge(samples, abi.MFLBM_FP64, abi.MFLBM_STRICT, tol=1e-5, interval=500,
                                   max_steps=40000)
    r32, _ = permeability.converge(samples, abi.MFLBM_FP32, tol=1e-5, interval=500, max_steps=40000)
    assert r64[0].get("converged", True) and r32[0].get("converged", True)
    assert r64[0]["k"] > 0
    assert abs(r32[0]["k"] - r64[0]["k"]) <= 0.01 * r64[0]["k"]
