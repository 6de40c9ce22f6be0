"""The oracle's output writers against the reference's own: after 20 steps of
every small case, in FP32 and FP64, the VTK files of types 1-3 (both
precision labels), the geometry VTK and the checkpoint written by the oracle
from its state have the SHA-256 of the files the reference's writers
produced for the same state (tests/golden/*.json, "outputs")."""
import json
from pathlib import Path

import pytest

import oracle_harness as H
from mflbm import abi, cases
from mflbm.geometry import read_dat

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
@pytest.mark.parametrize("kind", cases.SMALL_KINDS)
def test_oracle_writers_match_reference_files(kind, prec, tmp_path):
    case = cases.small_case(kind)
    gold = json.loads((GOLDEN / f"{case.name}_{H.suffix(prec)}.json").read_text())["outputs"]
    o = H.OracleState(case, prec, geometry=read_dat(GOLDEN / f"{case.name}.dat"))
    o.run(gold["step"])
    o.write_outputs(tmp_path, gold["step"])
    for name in H.OUTPUT_FILES:
        assert H.file_digest(tmp_path / name) == gold["sha256"][name], name
