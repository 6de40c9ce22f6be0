"""Batches and the autotuners (no reference counterpart; checked against the
library's own unbatched, untuned path, bit for bit):

  * a batch of contexts of different sizes and boundary conditions reaches
    exactly the states each context reaches when stepped alone, as one CUDA
    graph per step pair (two phases) or as persistent launches with grid
    barriers (single-phase samples);
  * a barrier wait that runs out returns MFLBM_E_TIMEOUT and leaves the
    library usable;
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


def _perm_ctx(n, porosity, seed, prec=abi.MFLBM_FP32, mode=abi.MFLBM_STRICT, **kw):
    from mflbm import lib
    return lib.setup_case(cases.permeability_sample(n, porosity, seed), prec, mode, **kw)[0]


SIZES = [(24, 0.5, 4100), (31, 0.4, 4101), (40, 0.6, 4102), (27, 0.35, 4103), (36, 0.65, 4104), (20, 0.55, 4105)]


@pytest.mark.parametrize("prec,mode,store", [(abi.MFLBM_FP32, abi.MFLBM_STRICT, abi.MFLBM_STORE_NATIVE),
                                             (abi.MFLBM_FP32, abi.MFLBM_FAST, abi.MFLBM_STORE_NATIVE),
                                             (abi.MFLBM_FP64, abi.MFLBM_STRICT, abi.MFLBM_STORE_NATIVE),
                                             (abi.MFLBM_FP32, abi.MFLBM_FAST, abi.MFLBM_STORE_F16)],
                         ids=["f32-strict", "f32-fast", "f64-strict", "f16-fast"])
def test_persistent_batch_equals_separate_runs(mflbm_lib, prec, mode, store):
    """Single-phase samples of uneven sizes: one persistent launch per up to
    100 steps (phases separated by grid barriers) reaches, for every sample,
    the state the sample reaches stepped alone, bit for bit."""
    from mflbm import lib
    solo = [_perm_ctx(*s, prec=prec, mode=mode, storage=store) for s in SIZES]
    grouped = [_perm_ctx(*s, prec=prec, mode=mode, storage=store) for s in SIZES]
    b = lib.Batch(grouped)
    b.run(1, 130)          # a graph-launched pair clears the start-up records, then 128 steps persistent
    assert b.options()["used_mode"] == abi.MFLBM_BATCH_PERSISTENT
    assert b.options()["grid"] > 1
    b.run(131, 72)
    for c in solo:
        c.run(1, 202)
    for s, g in zip(solo, grouped):
        assert _same(s, g)
    b.close()
    for c in solo + grouped:
        c.close()


def test_batch_modes_and_two_phase_fallback(mflbm_lib):
    from mflbm import lib
    a = [_perm_ctx(*s) for s in SIZES[:2]]
    b = lib.Batch(a)
    b.set_options(mode=abi.MFLBM_BATCH_GRAPH)
    b.run(1, 4)
    assert b.options()["used_mode"] == abi.MFLBM_BATCH_GRAPH
    b.set_options(mode=abi.MFLBM_BATCH_PERSISTENT)
    b.run(5, 4)
    assert b.options()["used_mode"] == abi.MFLBM_BATCH_PERSISTENT
    b.close()
    # a two-phase sample: persistent refused, AUTO falls back to the graph
    two = lib.Batch([_ctx("periodic_drop"), a[0]])
    two.set_options(mode=abi.MFLBM_BATCH_PERSISTENT)
    with pytest.raises(lib.MflbmError, match="no persistent launch"):
        two.run(1, 4)
    two.set_options(mode=abi.MFLBM_BATCH_AUTO)
    two.run(1, 4)
    assert two.options()["used_mode"] == abi.MFLBM_BATCH_GRAPH
    two.close()
    b2 = lib.Batch(a)
    with pytest.raises(lib.MflbmError, match="block"):
        b2.set_options(block=96)
    b2.close()
    for c in a:
        c.close()


def test_persistent_barrier_wait_runs_out(mflbm_lib):
    """A barrier wait bounded by 1 ns runs out: the run returns
    MFLBM_E_TIMEOUT instead of waiting, and the library stays usable (the
    contexts step again, and a fresh batch with the default bound gives the
    separate runs' results)."""
    from mflbm import lib
    ctxs = [_perm_ctx(*s) for s in SIZES]
    b = lib.Batch(ctxs)
    b.run(1, 4)                         # clears the start-up records
    assert b.options()["used_mode"] == abi.MFLBM_BATCH_PERSISTENT
    b.set_options(wait_limit_s=1e-9)
    with pytest.raises(lib.MflbmError) as e:
        b.run(5, 4)
    assert f"error {abi.MFLBM_E_TIMEOUT}" in str(e.value)
    b.close()
    for c in ctxs:
        c.run(9, 2)
        c.close()
    solo = [_perm_ctx(*s) for s in SIZES[:3]]
    grouped = [_perm_ctx(*s) for s in SIZES[:3]]
    g = lib.Batch(grouped)
    g.run(1, 20)
    for c in solo:
        c.run(1, 20)
    for s, q in zip(solo, grouped):
        assert _same(s, q)
    g.close()
    for c in solo + grouped:
        c.close()


def test_batch_autotune_keeps_results(mflbm_lib):
    from mflbm import lib
    solo = [_perm_ctx(*s) for s in SIZES[:4]]
    grouped = [_perm_ctx(*s) for s in SIZES[:4]]
    b = lib.Batch(grouped)
    b.run(1, 4)
    t = b.autotune(1)
    assert t["collide_block"] in (64, 128, 256) and t["tile_z"] in (1, 2)
    assert t["step_ms_after"] <= t["step_ms_before"] * 1.0001
    b.run(5, 16)
    for c in solo:
        c.run(1, 20)
    for s, g in zip(solo, grouped):
        assert _same(s, g)
    b.close()
    for c in solo + grouped:
        c.close()
