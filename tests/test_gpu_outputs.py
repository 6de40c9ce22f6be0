"""Output files written by the library (mflbm_write_vtk, mflbm_write_walls_vtk,
mflbm_write_checkpoint) and restart from a checkpoint (mflbm_read_checkpoint).

  * strict flavour, every small case, FP32 and FP64: after 20 steps the files
    are byte-identical to the reference's own writers' files for the same
    state (SHA-256 in tests/golden/*.json);
  * fast flavour: the files equal the oracle writers' files for the state the
    library downloads (the writers themselves add no rounding differences);
  * a checkpoint written by the library and one written in the reference's
    format by the oracle both restart to the reference's state at step 20;
  * a checkpoint of the wrong size is rejected with an error message.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
PRECS = [abi.MFLBM_FP32, abi.MFLBM_FP64]


def _golden(case, prec):
    return json.loads((GOLDEN / f"{case.name}_{H.suffix(prec)}.json").read_text())


def _lib_outputs(ctx, folder, ntime):
    folder = Path(folder)
    for name, (vtk_type, cmd) in H.VTK_FILES.items():
        ctx.write_vtk(vtk_type, folder / name, precision_cmd=cmd)
    ctx.write_walls_vtk(folder / "walls_bin.vtk")
    ctx.write_checkpoint(ntime, folder / "checkpoint")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("prec", PRECS, ids=["f32", "f64"])
@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_strict_files_match_reference(mflbm_lib, kind, prec, tmp_path):
    from mflbm import lib
    case = cases.small_case(kind)
    gold = _golden(case, prec)["outputs"]
    ctx, _ = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=read_dat(GOLDEN / f"{case.name}.dat"))
    ctx.run(1, gold["step"])
    _lib_outputs(ctx, tmp_path, gold["step"])
    for name in H.OUTPUT_FILES:
        assert H.file_digest(tmp_path / name) == gold["sha256"][name], name
    ctx.close()


@pytest.mark.parametrize("kind", ["velocity_convective", "pressure_pressure"])
def test_fast_files_match_oracle_writers(mflbm_lib, kind, tmp_path):
    from mflbm import lib
    case = cases.small_case(kind)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_FAST, geometry=geo)
    ctx.run(1, 20)
    (tmp_path / "lib").mkdir()
    (tmp_path / "orc").mkdir()
    _lib_outputs(ctx, tmp_path / "lib", 20)
    o = H.OracleState(case, abi.MFLBM_FP32, geometry=geo)
    for n, a in ctx.download().items():
        o.a[n][...] = a
    o.write_outputs(tmp_path / "orc", 20)
    for name in H.OUTPUT_FILES:
        assert H.file_digest(tmp_path / "lib" / name) == H.file_digest(tmp_path / "orc" / name), name
    ctx.close()


@pytest.mark.parametrize("prec", PRECS, ids=["f32", "f64"])
@pytest.mark.parametrize("kind", ["velocity_convective", "pressure_pressure"])
def test_restart_reaches_reference_state(mflbm_lib, kind, prec, tmp_path):
    from mflbm import lib
    case = cases.small_case(kind)
    gold = _golden(case, prec)
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, info = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=geo)
    ctx.run(1, 11)
    ctx.write_checkpoint(11, tmp_path / "lib_ckpt")
    ctx.close()
    o = H.OracleState(case, prec, geometry=geo)
    o.run(11)
    o.write_outputs(tmp_path, 11)   # 'checkpoint' in the reference's format
    for src in ("lib_ckpt", "checkpoint"):
        r, _ = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=geo)
        nt0 = r.read_checkpoint(tmp_path / src, W_in=o.a["W_in"])
        assert nt0 == 11
        r.run(nt0 + 1, 20 - nt0)
        d = r.download()
        for n, dg in gold["state"]["20"].items():
            assert _digest(d[n]) == dg, (src, n)
        r.close()


def test_truncated_checkpoint_is_rejected(mflbm_lib, tmp_path):
    from mflbm import lib
    case = cases.small_case("pressure_pressure")
    ctx, _ = lib.setup_case(case, abi.MFLBM_FP32, abi.MFLBM_STRICT, geometry=read_dat(GOLDEN / f"{case.name}.dat"))
    ctx.write_checkpoint(0, tmp_path / "ck")
    data = (tmp_path / "ck").read_bytes()
    (tmp_path / "short").write_bytes(data[:-4])
    with pytest.raises(lib.MflbmError, match="bytes, expected"):
        ctx.read_checkpoint(tmp_path / "short")
    ctx.close()
