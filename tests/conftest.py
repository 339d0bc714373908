import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Build libbcmg.so and the CPU oracle when missing or stale."""
    from bcmtools_gb300 import build as b
    b.build()
    from oracle import pyoracle
    if not pyoracle.LIB.exists() or any(
            p.stat().st_mtime > pyoracle.LIB.stat().st_mtime
            for p in (ROOT / "oracle").glob("bcm_oracle*")):
        pyoracle.build()
    yield


@pytest.fixture(scope="session")
def gpu_ok():
    import ctypes as C
    from bcmtools_gb300 import capi
    lib = capi.load()
    ctx = C.c_void_p()
    rc = lib.bcmg_ctx_create(C.byref(ctx), 0)
    if rc != 0:
        pytest.skip("no CUDA device")
    lib.bcmg_ctx_destroy(ctx)
    return True
