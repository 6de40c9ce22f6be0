"""mflbm_monitor_reduce_noalloc against mflbm_monitor_reduce, through the C ABI.

The no-allocation entry point keeps its partials in a static device array of
the library instead of memory allocated on the first call.  Two calls in a
row must each agree with the allocating entry point, and device memory must
not change across them.  The file is named to be collected last, so the
entry point is also exercised after every other GPU test has used the
library in the same process.
"""
import ctypes as C
from pathlib import Path

import pytest

from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
# both sides accumulate in FP64 over the same blocks; the tolerance only
# allows for a different block count on a device with another SM count
REL = 1e-12


def _free_device_bytes():
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("prec", [abi.MFLBM_FP32, abi.MFLBM_FP64], ids=["f32", "f64"])
def test_noalloc_matches_monitor_reduce(mflbm_lib, prec):
    from mflbm import lib
    case = cases.small_case("pressure_pressure")
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    ctx, _ = lib.setup_case(case, prec, abi.MFLBM_STRICT, geometry=geo)
    k = case.control_keys()
    nin, nout = int(k["n_exclude_inlet"]), int(k["n_exclude_outlet"])
    for first_step, steps in ((1, 10), (11, 2)):   # two post-even states
        ctx.run(first_step, steps)
        ref = ctx.monitor(nin, nout)
        before = _free_device_bytes()
        first = ctx.monitor_noalloc(nin, nout)
        second = ctx.monitor_noalloc(nin, nout)
        assert _free_device_bytes() == before
        for n, v in ref.items():
            assert first[n] == pytest.approx(v, rel=REL, abs=1e-300), (n, "first call")
            assert second[n] == pytest.approx(v, rel=REL, abs=1e-300), (n, "second call")
    ctx.close()
