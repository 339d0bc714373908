"""CPU: the reference's own RB-SOR benchmark path against the oracle.

oracle/_ref/refbench runs the reference's compiled code -- sor2's Solver
sweep (calcSorInBlock, examples/sor2/Solver.cpp:136-160) and Dirichlet
ghosts, the BlockManager ghost update through Scalar3DUpdater<double> -- on
the benchmark's kind of mesh (two-level sphere octree, 2:1 balanced, vc = 2,
Gaussian source).  The oracle's sor_run, which the GPU path is checked
against, must reproduce it bit for bit; the bench's CPU baseline times the
same binary.
"""
import numpy as np
import pytest

from bcmtools_gb300 import sor2_coef, workloads as W
from oracle import pyoracle as po
from oracle import refbench_io

pytestmark = pytest.mark.skipif(not refbench_io.available(),
                                reason="oracle/_ref/refbench not built (needs the reference)")


@pytest.mark.parametrize("n,level,iters", [(8, 2, 3), (16, 3, 2)])
def test_oracle_sor_matches_reference_benchmark_path(n, level, iters):
    w = W.two_level_sphere(n=n, vc=2, level=level)
    s = W.rhs_gaussian(w, seed=2, dtype=np.float64)
    _, f_ref = refbench_io.run(w.tree, n, 2, s, 1.8, threads=4, warmup=0, iters=iters)
    ld, nid, sf, _ = w.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, 2)
    bct, bcv = w.dirichlet(0.0)
    f = np.zeros(m.shape, np.float64)
    m.vc_update(f)
    m.dirichlet(f, bct, bcv, 0)
    m.sor_run(f, sor2_coef(w.tree.cell_sizes(n)), 1.8, 2, 1, iters, bct, bcv, 0, s=s)
    # edges and corners of the bricks: neither side writes them after f = 0
    assert np.array_equal(f, f_ref), int((f != f_ref).sum())
