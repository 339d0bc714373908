"""GPU: BiCGSTAB (plain and mixed precision) against the FP64 CPU oracle, and
the host-side failure paths (divergence status, memory budget)."""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import capi
from oracle import pyoracle as po
from tests.helpers import face_mask, outer_dirichlet, small_octree

pytestmark = pytest.mark.gpu


def problem(n=8, vc=1, level=2):
    tree = small_octree(periodic=(False, False, False), level=level, radius=0.3)
    bct, bcv = outer_dirichlet(tree, 0.0)
    cc = bg.laplace_coef(tree.cell_sizes(n))
    nb = tree.num_leaves
    rng = np.random.default_rng(21)
    ab = np.zeros((nb, n + 2 * vc, n + 2 * vc, n + 2 * vc))
    ab[:, vc:-vc, vc:-vc, vc:-vc] = rng.uniform(-1, 1, size=(nb, n, n, n))
    return tree, bct, bcv, cc, ab


def oracle_solution(tree, n, vc, bct, bcv, cc, ab):
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    ref = np.zeros_like(ab)
    it, res = m.bicgstab(ref, ab, 1.0, 2, 2000, 1e-13, bct, bcv, 0, cc=cc)
    assert it > 0 and res <= 1e-26
    return ref, it


def gpu_setup(tree, n, vc, bct, bcv, cc, dt):
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    x, b = bm.setDataClass(dt, vc), bm.setDataClass(dt, vc)
    op = bm.op_const(cc)
    return bm, x, b, op


def rel_err(got, ref, vc):
    g = got[:, vc:-vc, vc:-vc, vc:-vc].astype(np.float64)
    r = ref[:, vc:-vc, vc:-vc, vc:-vc]
    return np.linalg.norm(g - r) / np.linalg.norm(r)


def test_bicgstab_f64_matches_oracle(gpu_ok):
    n, vc = 8, 1
    tree, bct, bcv, cc, ab = problem(n, vc)
    ref, it_ref = oracle_solution(tree, n, vc, bct, bcv, cc, ab)
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f64")
    b.upload(ab)
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab(op, x, b, omega=1.0, n_pre=2, max_iter=2000, eps=1e-12)
    assert info.status == capi.SUCCESS and info.residual <= 1e-24
    assert abs(info.iterations - it_ref) <= max(3, it_ref // 10)
    assert rel_err(x.download(), ref, vc) < 1e-10


def two_level_15(n, vc):
    """15 blocks on two levels (level-jump faces of every kind)."""
    rg = bg.RootGrid(1, 1, 1, periodic=(False, False, False), root_length=1.0)
    tree = bg.Octree.build(rg, bg.Divider.sphere_surface((0.3, 0.3, 0.3), 0.1, 2), "Z")
    assert tree.num_leaves == 15
    bct, bcv = outer_dirichlet(tree, 0.0)
    cc = bg.laplace_coef(tree.cell_sizes(n))
    rng = np.random.default_rng(23)
    ab = np.zeros((15, n + 2 * vc, n + 2 * vc, n + 2 * vc))
    ab[:, vc:-vc, vc:-vc, vc:-vc] = rng.uniform(-1, 1, size=(15, n, n, n))
    return tree, bct, bcv, cc, ab


@pytest.mark.parametrize("n,vc", [(16, 1), (16, 2), (32, 1), (32, 2)])
def test_bicgstab_streamed_shapes_match_oracle(gpu_ok, n, vc):
    """16^3 and 32^3 blocks: A.p and A.s with their inner products, and the
    preconditioner's passes on 32^3 blocks, stream their planes through
    shared memory.  FP64 to 1e-12 must give the oracle's solution; FP32 to
    1e-6 must come within 1e-2 of it (|r|/|b| <= 1e-6 bounds the error by
    cond(A) * 1e-6)."""
    tree, bct, bcv, cc, ab = two_level_15(n, vc)
    ref, it_ref = oracle_solution(tree, n, vc, bct, bcv, cc, ab)
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f64")
    b.upload(ab)
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab(op, x, b, omega=1.0, n_pre=2, max_iter=2000, eps=1e-12)
    assert info.status == capi.SUCCESS and info.residual <= 1e-24
    # the iteration count to 1e-12 moves with the order of the sums across
    # blocks (the oracle's threaded sums vary from run to run by up to 10 %
    # here); the solution is the check
    assert abs(info.iterations - it_ref) <= max(5, it_ref // 4)
    assert rel_err(x.download(), ref, vc) < 1e-10
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f32")
    b.upload(ab.astype(np.float32))
    x.upload(np.zeros(ab.shape, np.float32))
    info = bm.bicgstab(op, x, b, omega=1.0, n_pre=2, max_iter=1000, eps=1e-6)
    assert info.status == capi.SUCCESS
    assert rel_err(x.download(), ref, vc) < 1e-2


def test_bicgstab_f32_error_vs_fp64_oracle(gpu_ok):
    n, vc = 8, 1
    tree, bct, bcv, cc, ab = problem(n, vc)
    ref, _ = oracle_solution(tree, n, vc, bct, bcv, cc, ab)
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f32")
    b.upload(ab.astype(np.float32))
    x.upload(np.zeros(ab.shape, np.float32))
    info = bm.bicgstab(op, x, b, omega=1.0, n_pre=2, max_iter=500, eps=1e-6)
    assert info.status == capi.SUCCESS
    # |r|/|b| <= 1e-6 bounds the error by cond(A) * 1e-6; measured ~1e-4 here
    assert rel_err(x.download(), ref, vc) < 2e-3


def test_bicgstab_mixed_reaches_1e10(gpu_ok):
    n, vc = 8, 1
    tree, bct, bcv, cc, ab = problem(n, vc, level=3)
    ref, _ = oracle_solution(tree, n, vc, bct, bcv, cc, ab)
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f64")
    b.upload(ab)
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab_mixed(op, x, b, omega=1.0, n_pre=2, max_inner=300, eps_inner=1e-4,
                             max_outer=30, eps=1e-10)
    assert info.status == capi.SUCCESS and info.true_residual <= 1e-10
    assert info.refinements >= 2
    assert rel_err(x.download(), ref, vc) < 1e-8


def test_bicgstab_mixed_reports_the_residual_of_its_x(gpu_ok):
    """Correction solves far too short to converge (3 iterations, halved on
    every refinement that does not help): the solve stops short of its target,
    and the residual it reports is the FP64 |b - Ax|/|b| of the x it leaves,
    which never got worse than the starting residual."""
    n, vc = 8, 1
    tree, bct, bcv, cc, ab = problem(n, vc, level=3)
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f64")
    b.upload(ab)
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab_mixed(op, x, b, omega=1.0, n_pre=2, max_inner=3, eps_inner=1e-8,
                             max_outer=12, eps=1e-14)
    assert info.status != capi.SUCCESS
    rr = bm.calc_r2(op, x, b)
    bb = bm.dot(b, b)
    assert abs(np.sqrt(rr / bb) - info.true_residual) <= 1e-9 * info.true_residual
    assert 0.0 < info.true_residual < 1.0


def test_nan_rhs_reports_divergence(gpu_ok):
    n, vc = 8, 1
    tree, bct, bcv, cc, ab = problem(n, vc)
    ab[0, vc + 1, vc + 1, vc + 1] = np.nan
    bm, x, b, op = gpu_setup(tree, n, vc, bct, bcv, cc, "f64")
    b.upload(ab)
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab(op, x, b, max_iter=50, eps=1e-10)
    assert info.status == capi.DIVERGED
    # the context stays usable after the failure
    b.upload(np.nan_to_num(ab))
    x.upload(np.zeros_like(ab))
    info = bm.bicgstab(op, x, b, max_iter=500, eps=1e-8)
    assert info.status == capi.SUCCESS


def test_memory_budget_rejects_over_allocation(gpu_ok):
    tree = small_octree(level=2)
    bm = bg.BlockManager(0)
    bm.register_octree(tree, 16)
    f = bm.setDataClass("f64", 2)
    used = bm.memory_in_use()
    assert used >= tree.num_leaves * 20 ** 3 * 8
    bm.set_memory_budget(used + 1000)
    with pytest.raises(bg.BcmgError) as e:
        bm.setDataClass("f64", 2)
    assert e.value.code == capi.MEMORY
    bm.destroy(f)
    assert bm.memory_in_use() == 0
    bm.setDataClass("f32", 1)


def test_argument_errors(gpu_ok):
    tree = small_octree(level=1)
    bm = bg.BlockManager(0)
    with pytest.raises(bg.BcmgError):
        bm.setDataClass("f32", 1)  # no blocks yet
    bm.register_octree(tree, 8)
    with pytest.raises(bg.BcmgError) as e:
        bm.setDataClass("f32", 5)  # vc > n/2 (DataClass.h:53)
    assert e.value.code == capi.USAGE
    f = bm.setDataClass("f32", 1)
    with pytest.raises(bg.BcmgError):
        bm.beginUpdateVC(f)  # prepareForVCUpdate missing
    bct = np.zeros((tree.num_leaves, 6), np.int32)
    bct[0, 0] = 7
    with pytest.raises(bg.BcmgError) as e:
        bm.set_boundary(bct, np.zeros((tree.num_leaves, 6)))
    assert e.value.code == capi.USAGE
    # Neumann faces are accepted; the SOR schemes reject them, as
    # sor1/Solver.cpp:214-221 does
    bct[0, 0] = bg.BC_NEUMANN
    bm.set_boundary(bct, np.zeros((tree.num_leaves, 6)))
    cc = bg.sor2_coef(tree.cell_sizes(8))
    with pytest.raises(bg.BcmgError) as e:
        bm.sor_run(f, cc, 1.0, form=1, n_inner=1, n_outer=1)
    assert e.value.code == capi.FAILURE
