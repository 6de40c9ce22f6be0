"""CUDA path against the CPU oracle.

Strict flavour (-fmad=false): every array bit-identical to the oracle (which
is bit-identical to the reference's own code) after N steps — geometry,
start-up fields, populations, phase field, normals, curvature and convective
buffers, in FP32 and FP64, through the graph-replayed path and the eager
path.  Fast flavour (FMA contraction): within the tolerances stated below.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
STATE = ["pdf", "phi", "cn_x", "cn_y", "cn_z", "c_norm", "curv", "f_convec_bc", "g_convec_bc", "phi_convec_bc"]
PRECS = [abi.MFLBM_FP32, abi.MFLBM_FP64]

# Fast-flavour tolerances (max abs difference against the oracle, populations
# and phase field are O(1)): FMA contraction changes the last bits of each
# operation; after 20 steps the drift stays within these bounds.
FAST_TOL = {abi.MFLBM_FP32: 2e-5, abi.MFLBM_FP64: 1e-12}


def _setup(kind, prec, mode):
    from mflbm import lib
    case = cases.small_case(kind)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, info = lib.setup_case(case, prec, mode, geometry=geo, want_host_geometry=True)
    o = H.OracleState(case, prec, geometry=geo)
    return case, ctx, info, o


def _diff(a, b):
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    return float(np.max(np.abs(a64 - b64))) if a.size else 0.0


@pytest.mark.parametrize("prec", PRECS, ids=["f32", "f64"])
@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_strict_is_bit_exact(mflbm_lib, kind, prec):
    case, ctx, info, o = _setup(kind, prec, abi.MFLBM_STRICT)
    g = info["geometry"]
    for n in ("walls", "walls_type", "s_nx", "s_ny", "s_nz"):
        assert g[n].tobytes() == o.a[n].tobytes(), f"geometry {n}"
    for n in ("num_solid_boundary_global", "num_fluid_boundary_global", "num_solid_boundary", "num_fluid_boundary",
              "pore_sum"):
        assert g["counts"][n] == getattr(o.counts, n), n
    done = 0
    for cp in [0, 1, 2, 11, 20]:
        if cp > done:
            ctx.run(done + 1, cp - done)
            o.run(cp - done)
            done = cp
        d = ctx.download()
        for n in STATE:
            assert d[n].tobytes() == o.a[n].tobytes(), f"{n} after {cp} steps (max diff {_diff(d[n], o.a[n])})"
    ctx.close()


@pytest.mark.parametrize("kind", ["velocity_convective", "periodic_drop", "closed_contact"])
def test_strict_is_bit_exact_on_odd_sizes(mflbm_lib, kind):
    """Odd extents on every axis: partial 2x2x2 bricks at the lattice ends
    (population bricks and the phase-field uniformity bricks of the normal
    pass)."""
    from mflbm import lib
    case = cases.small_case(kind, n=(21, 21, 23), seed=11)
    geo = case.geometry_bytes()
    ctx, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_STRICT, geometry=geo)
    o = H.OracleState(case, abi.MFLBM_FP32, geometry=geo)
    ctx.run(1, 30)
    o.run(30)
    d = ctx.download()
    for n in STATE:
        assert d[n].tobytes() == o.a[n].tobytes(), f"{n} after 30 steps (max diff {_diff(d[n], o.a[n])})"
    # the sparse sets of the last gradient pass: the interface nodes are the
    # nodes with c_norm != 0; the solid nodes it gave a non-zero normal are
    # those with one in the super-blocks it processed (all of them when it
    # processed every super-block)
    st = ctx.interface_stats()
    assert st["interface_nodes"] == np.count_nonzero(d["c_norm"]) > 0
    solid_nz = np.count_nonzero((d["cn_x"] != 0) | (d["cn_y"] != 0) | (d["cn_z"] != 0)) - st["interface_nodes"]
    sb = ctx.super_block_stats()
    if sb["processed"] == sb["total"]:
        assert st["solid_normals"] == solid_nz
    else:
        assert st["solid_normals"] <= solid_nz
    assert st["interface_nodes"] <= st["active_nodes"] <= 25 * 25 * 27
    ctx.close()


@pytest.mark.parametrize("kind", ["periodic_drop", "plate_drainage", "velocity_convective"])
def test_strict_long_run_with_moving_interface(mflbm_lib, kind):
    """500 steps with a moving interface, graph-replayed and per-step calls
    mixed: the interface set is rebuilt, and the solid phi, row masks and
    solid normals recomputed, every pass over the super-blocks where phi can
    have changed; every record, mask and solid value outside them must stay
    what the dense passes give, so stale entries would show up as
    differences."""
    case, ctx, info, o = _setup(kind, abi.MFLBM_FP32, abi.MFLBM_STRICT)
    sizes = []
    for first, count, eager in [(1, 60, False), (61, 30, True), (91, 210, False), (301, 40, True),
                                (341, 160, False)]:
        if eager:
            for nt in range(first, first + count):
                ctx.step(nt)
        else:
            ctx.run(first, count)
        o.run(count)
        d = ctx.download()
        for n in STATE:
            assert d[n].tobytes() == o.a[n].tobytes(), f"{n} after {first + count - 1} steps"
        st = ctx.interface_stats()
        assert st["interface_nodes"] == np.count_nonzero(d["c_norm"])
        sizes.append(st["interface_nodes"])
        # the super-block counts of the last pass (its list count alternates
        # between two counters across graph-replayed and per-step passes)
        sb = ctx.super_block_stats()
        assert 0 < sb["processed"] <= sb["total"] and sb["flagged"] <= sb["total"], sb
    assert min(sizes) > 0
    ctx.close()


@pytest.mark.parametrize("prec", PRECS, ids=["f32", "f64"])
def test_strict_eager_steps_and_upload(mflbm_lib, prec):
    """Per-step calls (mflbm_step) and a state uploaded from the host in the
    reference layouts (the drop-in's MemAllocate_multi_GPU path)."""
    from mflbm import lib
    case, ctx, info, o = _setup("velocity_convective", prec, abi.MFLBM_STRICT)
    o.run(5)
    ctx2 = lib.Context(info["params"])
    ctx2.upload_geometry(o.a["walls"], o.a["walls_type"], o.a["s_nx"], o.a["s_ny"], o.a["s_nz"])
    ctx2.upload_fields(**{n: o.a[n] for n in STATE + ["W_in"]})
    for nt in range(6, 13):
        ctx2.step(nt)
    o.run(7)
    d = ctx2.download()
    for n in STATE:
        assert d[n].tobytes() == o.a[n].tobytes(), n
    # the same download into the caller's buffers
    bufs = {n: np.full_like(o.a[n], np.nan) for n in STATE}
    d_into = ctx2.download(out=bufs)
    for n in STATE:
        assert d_into[n] is bufs[n] and bufs[n].tobytes() == o.a[n].tobytes(), n
    with pytest.raises(ValueError):
        ctx2.download(names=("phi",), out={"phi": np.zeros(3, dtype=o.a["phi"].dtype)})
    # upload without cn / c_norm / curv: recomputed on the device from phi
    ctx3 = lib.Context(info["params"])
    ctx3.upload_geometry(o.a["walls"], o.a["walls_type"], o.a["s_nx"], o.a["s_ny"], o.a["s_nz"])
    ctx3.upload_fields(pdf=o.a["pdf"], phi=o.a["phi"], W_in=o.a["W_in"], f_convec_bc=o.a["f_convec_bc"],
                       g_convec_bc=o.a["g_convec_bc"], phi_convec_bc=o.a["phi_convec_bc"])
    d3 = ctx3.download()
    for n in ("cn_x", "cn_y", "cn_z", "c_norm", "curv", "phi"):
        assert d3[n].tobytes() == o.a[n].tobytes(), n
    for c in (ctx, ctx2, ctx3):
        c.close()


@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_fast_fp64_within_tolerance(mflbm_lib, kind):
    case, ctx, info, o = _setup(kind, abi.MFLBM_FP64, abi.MFLBM_FAST)
    ctx.run(1, 20)
    o.run(20)
    d = ctx.download()
    for n, a, b in H.force_relevant_pairs(d, o.a):
        err = float(np.max(np.abs(a - b)))
        assert err <= FAST_TOL[abi.MFLBM_FP64], (n, err)
    ctx.close()


@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_fast_fp32_as_accurate_as_reference_fp32(mflbm_lib, kind):
    """FP32 with FMA contraction against the FP64 oracle, measured against the
    error of the reference's own FP32 arithmetic (the FP32 oracle) on the same
    FP64 oracle.

    FP32 rounding differences can flip a discrete decision at an isolated
    node: the 1e-6 cut-off of the normal, or the branch tests of the wetting
    secant iteration at a wall-adjacent interface node (observed at step 11 of
    the pressure/pressure case: one node's populations jump by 2e-3, and the
    jump then spreads over the neighbourhood).  The FP32 oracle flips at other
    nodes, or not at all, so a max-norm or high-percentile comparison between
    two FP32 programs on a 20 x 20 x 28 lattice is not meaningful.  Bounds:
      * median error of each quantity within 3x (+1e-7) of the FP32 oracle's
        (the bulk of the field carries rounding-level error only);
      * the mass of each component (conserved by the collision and the
        recolouring, so a local flip cannot move it) within 3x (+1e-6
        relative) of the FP32 oracle's error;
      * no error above 1e-2 anywhere (no amplification beyond a flip).
    The strict flavour, the same source without contraction, is checked
    bit-exact against the oracle elsewhere."""
    case, ctx, info, o32 = _setup(kind, abi.MFLBM_FP32, abi.MFLBM_FAST)
    o64 = H.OracleState(case, abi.MFLBM_FP64, geometry=o32.geometry)
    ctx.run(1, 20)
    o32.run(20)
    o64.run(20)
    d = ctx.download()
    ref32 = {n: v for n, v, _ in H.force_relevant_pairs(o32.a, o64.a)}
    for n, a, b in H.force_relevant_pairs(d, o64.a):
        err_gpu, err_ref = np.abs(a - b).ravel(), np.abs(ref32[n] - b).ravel()
        q_gpu, q_ref = float(np.median(err_gpu)), float(np.median(err_ref))
        assert q_gpu <= 3 * q_ref + 1e-7, (n, "median", q_gpu, q_ref)
        assert float(err_gpu.max()) <= 1e-2, (n, "max", float(err_gpu.max()), float(err_ref.max()))

    def component_masses(pdf):
        f = pdf.reshape(38, -1).astype(np.float64)
        return float(f[:19].sum()), float(f[19:].sum())

    for m_gpu, m_ref, m64 in zip(component_masses(d["pdf"]), component_masses(o32.a["pdf"]),
                                 component_masses(o64.a["pdf"])):
        assert abs(m_gpu - m64) <= 3 * abs(m_ref - m64) + 1e-6 * abs(m64), (m_gpu, m_ref, m64)
    ctx.close()


@pytest.mark.parametrize("prec", PRECS, ids=["f32", "f64"])
def test_monitor_reductions_match_oracle(mflbm_lib, prec):
    case, ctx, info, o = _setup("pressure_pressure", prec, abi.MFLBM_STRICT)
    ctx.run(1, 10)
    o.run(10)
    k = case.control_keys()
    m = ctx.monitor(int(k["n_exclude_inlet"]), int(k["n_exclude_outlet"]))
    mo = o.monitor()
    # both sides sum in FP64; the oracle sums serially (~1e6 terms for
    # total_mass), the device as a tree, so they agree to ~1e-10 relative
    for n, v in mo.items():
        assert m[n] == pytest.approx(v, rel=1e-10, abs=1e-14), n
    ctx.close()


def test_drainage_48x48x64_fp64_2000_steps(mflbm_lib):
    """The reference's FP64 parity workload: drainage in a 48 x 48 x 64 sphere
    pack, 2000 steps.  Strict: bit-exact.  Fast: phase field within 1e-9,
    populations within 1e-11, saturation within 1e-12 relative."""
    from mflbm import lib
    case = cases.drainage_48x48x64()
    geo = case.geometry_bytes()
    o = H.OracleState(case, abi.MFLBM_FP64, geometry=geo)
    o.run(2000)
    ms = o.macro()
    mo = o.monitor()
    for mode in (abi.MFLBM_STRICT, abi.MFLBM_FAST):
        ctx, info = lib.setup_case(case, abi.MFLBM_FP64, mode, geometry=geo)
        ctx.run(1, 2000)
        d = ctx.download()
        m = ctx.monitor(2, 2)
        if mode == abi.MFLBM_STRICT:
            for n in STATE:
                assert d[n].tobytes() == o.a[n].tobytes(), n
        else:
            assert _diff(d["phi"], o.a["phi"]) < 1e-9
            assert _diff(d["pdf"], o.a["pdf"]) < 1e-11
            assert m["saturation"] == pytest.approx(mo["saturation"], rel=1e-12)
        ctx.close()
    assert 0.0 < mo["saturation"] < 1.0
    assert np.isfinite(ms["w"]).all()


def test_graph_replays_refresh_exported_arrays(mflbm_lib):
    """Steps that only replay the captured step-pair graph still refresh the
    reference-layout gradient arrays a later download exports."""
    case, ctx, info, o = _setup("velocity_convective", abi.MFLBM_FP32, abi.MFLBM_STRICT)
    ctx.run(1, 4)        # captures the pair graph
    ctx.download()       # exports the arrays
    ctx.run(5, 4)        # graph replays only
    o.run(8)
    d = ctx.download()
    for n in ("cn_x", "c_norm", "curv", "pdf", "phi"):
        assert d[n].tobytes() == o.a[n].tobytes(), n
    ctx.close()


@pytest.mark.parametrize("tile", [(1, 1, 1), (2, 2, 2), (32, 32, 2), (4, 8, 1)], ids=lambda t: "x".join(map(str, t)))
@pytest.mark.parametrize("kind,n", [("velocity_convective", (20, 20, 28)), ("periodic_drop", (21, 21, 23))])
def test_strict_bit_exact_with_tile_shapes(mflbm_lib, kind, n, tile):
    """Other population tile shapes: the populations and the collision
    records move exactly when the shape changes (before the first step and
    in the middle of a run), so the state stays bit-identical to the oracle;
    the per-slice monitor profile (one block per layer of tiles) equals the
    default shape's to FP64 rounding."""
    from mflbm import lib
    case = cases.small_case(kind, n=n, seed=11 if n != (20, 20, 28) else 7)
    geo = read_dat(GOLDEN / f"{case.name}.dat") if n == (20, 20, 28) else case.geometry_bytes()
    ctx, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_STRICT, geometry=geo)
    ref, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_STRICT, geometry=geo)
    o = H.OracleState(case, abi.MFLBM_FP32, geometry=geo)
    ctx.set_tuning(tile=tile)
    assert (ctx.get_tuning()["tile_x"], ctx.get_tuning()["tile_y"], ctx.get_tuning()["tile_z"]) == tile
    for first, count, switch in [(1, 10, (8, 4, 2)), (11, 10, tile)]:
        ctx.run(first, count)
        ref.run(first, count)
        o.run(count)
        d = ctx.download()
        for name in STATE:
            assert d[name].tobytes() == o.a[name].tobytes(), f"{name} after {first + count - 1} steps"
        # FP64 sums over the same nodes in another order (the list follows the layout)
        p, e = ctx.monitor_profile()
        pr, er = ref.monitor_profile()
        for row in p:
            assert np.allclose(p[row], pr[row], rtol=1e-12, atol=1e-14), row
        for key in e:
            assert e[key] == pytest.approx(er[key], rel=1e-12, abs=1e-14), key
        ctx.set_tuning(tile=switch)
    ctx.close()
    ref.close()
