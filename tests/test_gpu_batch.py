"""GPU: batched instances (bcmtools_gb300.batch) -- each instance's values
in the batch equal the values it gets alone, bit for bit."""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import workloads as W
from bcmtools_gb300.batch import Batch
from tests.helpers import assert_bitexact

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [8, 16, 32])
def test_batch_equals_alone(gpu_ok, n):
    ws = [W.random_instance(s, min_blocks=8, max_blocks=200, sizes=(n,)) for s in (11, 12, 13)]
    seeds = [101, 102, 103]
    iters = 6
    batch = Batch(ws)
    batch.set_dirichlet(0.0)
    op = batch.laplace_op()
    x, b = batch.bm.setDataClass("f32", 1), batch.bm.setDataClass("f32", 1)
    batch.fill_rhs(b, seeds)
    x.fill(0.0)
    batch.bm.imposeBoundaryCondition(x)
    batch.bm.jacobi_run(op, x, b, 0.9, iters)
    xb = x.download()
    for k, w in enumerate(ws):
        bm = bg.BlockManager(0)
        bm.register_octree(w.tree, n)
        t, v = w.dirichlet(0.0)
        bm.set_boundary(t, v, bg.DIRICHLET_SOR)
        op1 = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(n)))
        x1, b1 = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
        b1.fill(0.0)
        b1.fill_random(seeds[k])
        assert_bitexact(b1.download(), batch.instance(b.download(), k), what=f"rhs {k}")
        x1.fill(0.0)
        bm.imposeBoundaryCondition(x1)
        bm.jacobi_run(op1, x1, b1, 0.9, iters)
        assert_bitexact(x1.download(), batch.instance(xb, k), what=f"instance {k} n={n}")
