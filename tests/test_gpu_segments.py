"""GPU: independent systems batched into one mesh (bcmg_set_segments).

Instances of different block counts are registered as one block set, each a
segment; one BiCGSTAB call (FP32, FP64) and one mixed-precision call then
advance all of them with every launch.  Each instance's scalars, residuals
and convergence test are its own, so its result must be the one it gets
solved alone: the same iteration count and the same field bit for bit.
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import workloads as W
from bcmtools_gb300.batch import Batch

pytestmark = pytest.mark.gpu

SEEDS = [1000, 1001, 1002]


def _instances(n=8):
    ws = [W.random_instance(s, min_blocks=16, max_blocks=80, sizes=(n,)) for s in SEEDS]
    return [w for w in ws]


def _solve_alone(w, seed, dt, mixed):
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    t, v = w.dirichlet(0.0)
    bm.set_boundary(t, v, bg.DIRICHLET_SOR)
    op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
    x, b = bm.setDataClass(dt, w.vc), bm.setDataClass(dt, w.vc)
    b.fill(0.0)
    b.fill_random(seed)
    x.fill(0.0)
    bm.imposeBoundaryCondition(x)
    if mixed:
        info = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=60, eps_inner=1e-2,
                                 max_outer=20, eps=1e-9)
    else:
        info = bm.bicgstab(op, x, b, omega=0.8, n_pre=2, max_iter=400, eps=1e-6)
    return info, x.download()


@pytest.mark.parametrize("n", [8, 32])
@pytest.mark.parametrize("dt,mixed", [("f32", False), ("f64", False), ("f64", True)])
def test_segments_match_solving_alone(gpu_ok, dt, mixed, n):
    """32^3 blocks take the streamed kernels, with p's and s's updates made
    by their preconditioner's first pass (a finished segment's blocks
    skipped there too)."""
    ws = _instances(n)
    batch = Batch(ws)
    batch.set_dirichlet(0.0)
    op = batch.laplace_op()
    bm = batch.bm
    x, b = bm.setDataClass(dt, 1), bm.setDataClass(dt, 1)
    batch.fill_rhs(b, SEEDS)
    x.fill(0.0)
    bm.imposeBoundaryCondition(x)
    batch.set_segments()
    if mixed:
        infos = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=60, eps_inner=1e-2,
                                  max_outer=20, eps=1e-9)
    else:
        infos = bm.bicgstab(op, x, b, omega=0.8, n_pre=2, max_iter=400, eps=1e-6)
    got = x.download()
    assert len(infos) == len(ws)
    for k, w in enumerate(ws):
        info, ref = _solve_alone(w, SEEDS[k], dt, mixed)
        assert infos[k].status == info.status == 0, (k, infos[k].status, info.status)
        assert infos[k].iterations == info.iterations, (k, infos[k].iterations, info.iterations)
        assert infos[k].refinements == info.refinements
        assert np.array_equal(batch.instance(got, k), ref), k


def test_segments_reject_shared_faces(gpu_ok):
    """A face joining two segments would couple their systems: refused."""
    w = W.plain_poisson(n=8, vc=1, level=1)
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    with pytest.raises(bg.BcmgError):
        bm.set_segments([0, 4, w.nb])
