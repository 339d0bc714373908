"""GPU: bcmg_dot_noalloc, the inner product that allocates nothing.

It exists for callers that cannot call cudaMalloc: host code inside an
application or framework that owns every device allocation through its own
pool.  Its per-block scratch is a fixed array inside the library instead of
a per-context buffer, so the test checks it through the C ABI against
bcmg_dot (same kernels, so the values must agree to 1e-12 relative -- in
practice bit for bit) on two calls in a row, in FP32 and FP64, plus the size
limits.  The file sorts last so that a run stopping at the first failure has
run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import capi
from tests.helpers import small_octree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_noalloc_dot_matches_dot(gpu_ok, dt):
    torch = pytest.importorskip("torch")
    n, vc = 8, 2
    tree = small_octree(level=3, radius=0.3)
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    fields = [bm.setDataClass(dt, vc) for _ in range(4)]
    rng = np.random.default_rng(17)
    for f in fields:
        f.upload(rng.uniform(-1, 1, size=f.shape).astype(f.dtype))
    lib = capi.load()
    code = capi.F32 if dt == "f32" else capi.F64
    torch.cuda.set_device(0)
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    for call, (x, y) in enumerate([(fields[0], fields[1]), (fields[2], fields[3])]):
        ref = bm.dot(x, y)
        px, stride, _ = x.layout()
        py, _, _ = y.layout()
        rc = lib.bcmg_dot_noalloc(code, px, py, bm.nb, n, n, n, vc, stride,
                                  out.data_ptr() + 8 * call, None)
        assert rc == capi.SUCCESS
        torch.cuda.synchronize()
        got = float(out[call].item())
        assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref)), (call, got, ref)


def test_noalloc_dot_rejects_too_many_blocks(gpu_ok):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    buf = torch.zeros(64, dtype=torch.float32, device="cuda:0")
    p = buf.data_ptr()
    rc = lib.bcmg_dot_noalloc(capi.F32, p, p, 65536 + 1, 2, 2, 2, 1, 64, out.data_ptr(), None)
    assert rc == capi.SCRATCH_LIMIT
    rc = lib.bcmg_dot_noalloc(capi.F32, p, p, 1, 2, 2, 2, 1, 8, out.data_ptr(), None)
    assert rc == capi.USAGE  # block stride smaller than a 4^3 brick
    # a brick plane beyond int32 elements is refused before any launch
    rc = lib.bcmg_dot_noalloc(capi.F32, p, p, 1, 50000, 50000, 2, 1, 2**40, out.data_ptr(), None)
    assert rc == capi.USAGE
