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
