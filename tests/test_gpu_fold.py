"""GPU: boundary folding of a coefficient-brick operator
(bcmg_op_fold_boundary; SolverTest bca.f90:12-394, LocalScalar3D.h:260-285)
through the C ABI, bit-exact against the oracle, then Jacobi iterations with
the folded operator bit-exact against the oracle's."""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import capi
from oracle import pyoracle as po
from tests.helpers import assert_bitexact, face_mask, outer_dirichlet, small_octree

pytestmark = pytest.mark.gpu


def rand(shape, dt, seed):
    return np.random.default_rng(seed).uniform(-1, 1, size=shape).astype(dt)


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("n,vc", [(8, 1), (16, 2)])
def test_fold_then_jacobi_match_oracle(gpu_ok, dt, n, vc):
    tree = small_octree(periodic=(False, True, False), level=2, radius=0.3)
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    bct, bcv = outer_dirichlet(tree, 0.3, periodic=(False, True, False))
    bct[:, 4:6] = np.where(bct[:, 4:6] != 0, bg.BC_NEUMANN, 0)
    bcv[:, 4:6] = np.random.default_rng(6).uniform(-0.05, 0.05, size=(bct.shape[0], 2))
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    x, b = bm.setDataClass(dt, vc), bm.setDataClass(dt, vc)
    npdt = x.dtype
    A = [rand(x.shape, npdt, 30 + k) for k in range(7)]
    A[0] = (np.abs(A[0]) + 6.0).astype(npdt)
    fs = [bm.setDataClass(dt, vc) for _ in range(7)]
    for fk, ak in zip(fs, A):
        fk.upload(ak)
    op = bm.op_fields(fs)
    ab = np.zeros(x.shape, npdt)
    ab[:, vc:-vc, vc:-vc, vc:-vc] = rand((x.shape[0], n, n, n), npdt, 40)
    b.upload(ab)
    bm.fold_boundary(op, b)
    refA = [a.copy() for a in A]
    refb = ab.copy()
    m.fold(refA, refb, bct, bcv)
    for k in range(7):
        assert_bitexact(fs[k].download(), refA[k], what=f"folded A[{k}]")
    assert_bitexact(b.download(), refb, what="folded b")
    assert not np.array_equal(refb, ab)

    a0 = rand(x.shape, npdt, 41)
    x.upload(a0)
    iters = 4
    bm.jacobi_run(op, x, b, 0.9, iters)
    ref = a0.copy()
    x1 = np.zeros_like(ref)
    for _ in range(iters):
        m.jacobi(x1, ref, refb, 0.9, fields=refA)
        ref[:, vc:-vc, vc:-vc, vc:-vc] = x1[:, vc:-vc, vc:-vc, vc:-vc]
        m.vc_update(ref)
        m.dirichlet(ref, bct, bcv, 0)
    assert_bitexact(x.download(), ref, face_mask(n, vc), f"jacobi on the folded operator {dt}")


def test_fold_needs_coefficient_fields(gpu_ok):
    tree = small_octree(level=1)
    bm = bg.BlockManager(0)
    bm.register_octree(tree, 8)
    b = bm.setDataClass("f32", 1)
    op = bm.op_const(bg.laplace_coef(tree.cell_sizes(8)))
    with pytest.raises(bg.BcmgError) as e:
        bm.fold_boundary(op, b)
    assert e.value.code == capi.USAGE
