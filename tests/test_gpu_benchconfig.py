"""GPU parity at the benchmark configurations, through the C ABI.

The timed kernels on the meshes the bench times them on, against the oracle
(itself pinned to the reference's compiled code, tests/test_refbench_cpu.py
and tests/test_oracle_golden.py):

* the two-level sphere (4432 blocks of 16^3, vc = 2, 18.2 M cells), 10
  red-black SOR iterations at omega = 1.8 with the Gaussian source through
  the default fused kernel (pull form, one CTA per block, packed source):
  FP64 bit-exact; FP32 within 1e-6 relative (normwise) after one sweep and
  1e-5 after ten;
* flat level 5 (32768 blocks of 16^3, vc = 1, 134 M cells), 3 fused Jacobi
  sweeps with the ghost update and Dirichlet ghosts (pull form, one CTA per
  block): bit-exact;
* the mixed-precision benchmark's right-hand side generator against its host
  copy (the FP64 CPU solution stored in tests/golden is of that system).
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import workloads as W
from oracle import pyoracle as po
from tests.helpers import assert_bitexact, assert_close_normwise, face_mask

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    w = W.two_level_sphere(n=16, vc=2)
    assert w.nb == 4432
    bct, bcv = w.dirichlet(0.0)
    coef = bg.sor2_coef(w.tree.cell_sizes(w.n))
    return w, bct, bcv, coef


def _c2_gpu(w, bct, bcv, coef, dt, s_host, iters):
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    f, s = bm.setDataClass(dt, w.vc), bm.setDataClass(dt, w.vc)
    bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
    s.upload(s_host)
    f.fill(0.0)
    bm.imposeBoundaryCondition(f)
    bm.sor_run(f, coef, 1.8, form=2, n_inner=1, n_outer=iters, s=s)
    return f.download()


def _c2_oracle(w, bct, bcv, coef, s_host, iters):
    ld, nid, sf, _ = w.neighbors()
    m = po.OracleMesh(ld, nid, sf, w.n, w.vc)
    ref = np.zeros(m.shape, s_host.dtype)
    m.vc_update(ref)
    m.dirichlet(ref, bct, bcv, 0)
    m.sor_run(ref, coef, 1.8, 2, 1, iters, bct, bcv, 0, s=s_host)
    return ref


def test_c2_sor_f64_full_mesh_bitexact(gpu_ok, c2):
    w, bct, bcv, coef = c2
    s_host = W.rhs_gaussian(w, seed=2, dtype=np.float64)
    got = _c2_gpu(w, bct, bcv, coef, "f64", s_host, 10)
    ref = _c2_oracle(w, bct, bcv, coef, s_host, 10)
    assert_bitexact(got, ref, face_mask(w.n, w.vc), "C2 SOR f64, 10 iterations")


@pytest.mark.parametrize("iters,tol", [(1, 1e-6), (10, 1e-5)])
def test_c2_sor_f32_full_mesh_within_tolerance(gpu_ok, c2, iters, tol):
    w, bct, bcv, coef = c2
    s_host = W.rhs_gaussian(w, seed=2, dtype=np.float32)
    got = _c2_gpu(w, bct, bcv, coef, "f32", s_host, iters)
    ref = _c2_oracle(w, bct, bcv, coef, s_host, iters)
    assert_close_normwise(got, ref, tol, face_mask(w.n, w.vc), f"C2 SOR f32, {iters} sweeps")


def test_c1_level5_fused_jacobi_bitexact(gpu_ok):
    w = W.plain_poisson(n=16, vc=1, level=5)
    assert w.nb == 32768
    bct, bcv = w.dirichlet(0.0)
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    x, b = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
    bh = W.rhs_uniform(w, seed=1, dtype=np.float32)
    b.upload(bh)
    cc = bg.laplace_coef(w.tree.cell_sizes(w.n))
    op = bm.op_const(cc)
    x.fill(0.0)
    bm.imposeBoundaryCondition(x)
    bm.jacobi_run(op, x, b, 1.0, 3)
    got = x.download()
    ld, nid, sf, _ = w.neighbors()
    m = po.OracleMesh(ld, nid, sf, w.n, 1)
    ref = np.zeros(m.shape, np.float32)
    m.vc_update(ref)
    m.dirichlet(ref, bct, bcv, 0)
    x1 = np.zeros_like(ref)
    for _ in range(3):
        m.jacobi(x1, ref, bh, 1.0, cc=cc)
        ref[:, 1:-1, 1:-1, 1:-1] = x1[:, 1:-1, 1:-1, 1:-1]
        m.vc_update(ref)
        m.dirichlet(ref, bct, bcv, 0)
    assert_bitexact(got, ref, face_mask(w.n, 1), "C1 level 5, 3 fused Jacobi sweeps")


def test_c3_rhs_generator_matches_host_copy(gpu_ok):
    """fill_random on the device gives the host copy the FP64 CPU solution
    of the mixed-precision benchmark was computed with (checked on a
    smaller mesh of the same generator: the values depend only on the seed,
    the block and the cell)."""
    w = W.points_level5(n=8, level=3)
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    for dt, npdt in (("f64", np.float64), ("f32", np.float32)):
        b = bm.setDataClass(dt, 1)
        b.fill(0.0)
        b.fill_random(3)
        assert_bitexact(b.download(), W.rhs_fill_random(w, 3, npdt), what=f"fill_random {dt}")
