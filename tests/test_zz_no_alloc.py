"""mflbm_monitor_reduce_noalloc against mflbm_monitor_reduce, through the C ABI.

The no-allocation entry point keeps its partials in a static device array of
the library instead of memory allocated on the first call.  It serves callers
that cannot allocate device memory mid-run: a lattice sized to fill the GPU
leaves no room for the allocating entry point's first-call cudaMalloc, and
cudaMalloc / cudaFree synchronise the whole device.

After a run of steps, the no-allocation call comes first (so that it, not the
allocating call, refreshes the exported reference-layout arrays); then the
allocating entry point and a second no-allocation call follow.  Both entry
points group the FP64 partial sums over the same blocks, so all three results
must be bit-identical.  Neither the device's free memory nor the default
stream-ordered memory pool may change across the two no-allocation calls.

The file is named to be collected last, so the entry point is also exercised
after every other GPU test has used the library in the same process.
"""
import ctypes as C
from pathlib import Path

import pytest

from mflbm import abi, cases
from mflbm.geometry import read_dat

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
CUDA_MEMPOOL_ATTR_USED_MEM_CURRENT = 7   # cudaMemPoolAttrUsedMemCurrent
CUDA_MEMPOOL_ATTR_RESERVED_MEM_CURRENT = 5


def _device_memory_state():
    """(free device bytes, default pool used bytes, default pool reserved bytes)."""
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    dev = C.c_int()
    assert rt.cudaGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    used, reserved = C.c_uint64(), C.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, CUDA_MEMPOOL_ATTR_USED_MEM_CURRENT, C.byref(used)) == 0
    assert rt.cudaMemPoolGetAttribute(pool, CUDA_MEMPOOL_ATTR_RESERVED_MEM_CURRENT, C.byref(reserved)) == 0
    return free.value, used.value, reserved.value


CASES = [
    (abi.MFLBM_FP32, abi.MFLBM_STORE_NATIVE),
    (abi.MFLBM_FP64, abi.MFLBM_STORE_NATIVE),
    (abi.MFLBM_FP32, abi.MFLBM_STORE_F16),
    (abi.MFLBM_FP32, abi.MFLBM_STORE_BF16),
]


@pytest.mark.parametrize("prec,storage", CASES, ids=["f32", "f64", "f16-storage", "bf16-storage"])
def test_noalloc_matches_monitor_reduce(mflbm_lib, prec, storage):
    from mflbm import lib
    case = cases.small_case("pressure_pressure")
    geo = read_dat(GOLDEN / f"{case.name}.dat")
    mode = abi.MFLBM_STRICT if storage == abi.MFLBM_STORE_NATIVE else abi.MFLBM_FAST
    ctx, _ = lib.setup_case(case, prec, mode, geometry=geo, storage=storage)
    k = case.control_keys()
    nin, nout = int(k["n_exclude_inlet"]), int(k["n_exclude_outlet"])
    for first_step, steps in ((1, 10), (11, 2)):   # two post-even states
        ctx.run(first_step, steps)
        before = _device_memory_state()
        first = ctx.monitor_noalloc(nin, nout)      # first call after the steps
        second = ctx.monitor_noalloc(nin, nout)
        assert _device_memory_state() == before, "device memory changed across the no-allocation calls"
        ref = ctx.monitor(nin, nout)
        assert set(first) == set(ref)
        for n, v in ref.items():
            assert first[n] == v, (n, "first call", first[n], v)
            assert second[n] == v, (n, "second call", second[n], v)
    ctx.close()
