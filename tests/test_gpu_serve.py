"""GPU: served solves -- every request's solution in the concurrent mix is
the one it gets alone, bit for bit, and meets its residual target."""
import numpy as np
import pytest

from bcmtools_gb300 import capi, serve
from tests.helpers import assert_bitexact

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(gpu_ok):
    reqs = serve.poisson_stream(6, 500.0, seed=7, cells=(3e4, 2e5), sizes=(8, 16),
                                levels=(2, 3), eps=1e-8)
    mixed = serve.Server(budget_bytes=2e9, workers=3).run(reqs, keep=True)
    assert len(mixed) == len(reqs)
    for r, m in zip(reqs, mixed):
        assert m.status == capi.SUCCESS and m.residual <= 1e-8
        info, nb, cells, x = serve.solve_alone(r, keep=True)
        assert info.iterations == m.iterations and nb == m.blocks
        assert_bitexact(m.x, x, what=f"request {r.rid}")


def test_batched_served_results_equal_alone(gpu_ok):
    """Continuous batching: requests solved as segments of shared batches
    (several per batch, batches running concurrently) get the solution they
    get alone, bit for bit, with the same iteration and refinement counts."""
    reqs = serve.poisson_stream(10, 2000.0, seed=11, cells=(2e4, 3e5), sizes=(8, 16),
                                levels=(2, 3), eps=1e-8)
    srv = serve.BatchServer(budget_bytes=4e9, workers=2, size_ratio=8.0)
    mixed = srv.run(reqs, keep=True)
    assert len(mixed) == len(reqs)
    assert max(m.batch for m in mixed) >= 2  # some requests shared a batch
    for r, m in zip(reqs, mixed):
        assert m.status == capi.SUCCESS and m.residual <= 1e-8
        info, nb, cells, x = serve.solve_alone(r, keep=True)
        assert info.iterations == m.iterations and info.refinements == m.refinements
        assert nb == m.blocks
        assert_bitexact(m.x, x, what=f"request {r.rid}")


def test_plain_path_solves_to_target_and_agrees_with_mixed(gpu_ok):
    """The plain path (FP64 BiCGSTAB, one request at a time) meets each
    request's 1e-8 target, and its solution agrees with the mixed-precision
    one to what two 1e-8 residuals allow (their difference is bounded by the
    system's condition number, a few thousand here, times 2e-8)."""
    reqs = serve.poisson_stream(3, 500.0, seed=13, cells=(3e4, 2e5), sizes=(8, 16),
                                levels=(2, 3), eps=1e-8)
    for r in reqs:
        ip, nbp, _, xp = serve.solve_plain(r, keep=True)
        im, nbm, _, xm = serve.solve_alone(r, keep=True)
        assert ip.status == capi.SUCCESS and ip.true_residual <= 1e-8 and ip.refinements == 0
        assert im.status == capi.SUCCESS and nbp == nbm
        d = np.linalg.norm(xp.astype(np.float64) - xm) / np.linalg.norm(xm)
        assert d < 1e-3, (r.rid, d)
