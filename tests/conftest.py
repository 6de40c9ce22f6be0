import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (str(REPO / "mf-lbm-cuda_gb300"), str(REPO / "tests"), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def mflbm_lib():
    """Build (if stale) and load libmflbm.so."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mflbm_build", REPO / "mf-lbm-cuda_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    from mflbm import lib
    return lib.load()
