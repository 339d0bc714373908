import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # Build libbcmg.so and the CPU oracle when missing or stale, before the
    # test modules (which import the package) are collected.
    import __graft_entry__
    __graft_entry__._build_module().build()
    from oracle import pyoracle
    if not pyoracle.LIB.exists() or any(
            p.stat().st_mtime > pyoracle.LIB.stat().st_mtime
            for p in (ROOT / "oracle").glob("bcm_oracle*")):
        pyoracle.build()


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
