"""CPU: the oracle's Jacobi and BiCGSTAB against the reference's ILS3D.

oracle/_ref/refils3d runs the reference's own ILS3D::Jacobi and
ILS3D::BiCGSTAB (examples/SolverTest/ILS3D.h:478-529, 663-844, compiled from
the reference's header) over the reference's BlockManager and
Scalar3DUpdater<double>, with the blas.f90 loop bodies taken from the oracle
(the image has no Fortran compiler).  On a two-level octree with a
boundary-folded coefficient-brick operator (bca.f90 via the oracle's fold),
the oracle's restated solvers must give the reference's iteration count,
residual and field bit for bit: that pins the solvers' step order, scalar
recurrences, reductions across blocks and convergence test, which the GPU
solvers are in turn checked against.  Single-threaded on both sides, so that
every sum over blocks runs in block order.  One difference is by design: at
the iteration limit ILS3D's loop variable is left at countMax + 1 (the value
that ended its for loop), where the oracle and the library report the
iterations done, countMax.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import bcmtools_gb300 as bg
from oracle import pyoracle as po
from tests.helpers import outer_dirichlet, small_octree

BIN = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "refils3d"
pytestmark = pytest.mark.skipif(not BIN.exists(), reason="oracle/_ref/refils3d not built")


def _system(n=8, vc=1, seed=3):
    tree = small_octree(periodic=(False, False, False), level=2, radius=0.3)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    bct, bcv = outer_dirichlet(tree, 0.0)
    cc = bg.laplace_coef(tree.cell_sizes(n))
    fields = [np.empty(m.shape) for _ in range(7)]
    for c in range(7):
        fields[c][...] = cc[:, c][:, None, None, None]
    rng = np.random.default_rng(seed)
    b = np.zeros(m.shape)
    b[:, vc:-vc, vc:-vc, vc:-vc] = rng.uniform(-1, 1, size=(tree.num_leaves, n, n, n))
    m.fold(fields, b, bct, bcv)
    return tree, m, fields, b, bct, bcv


def _run_reference(tree, n, vc, fields, b, x, mode, n_pre, max_iter, omega, eps, tmp):
    rg = tree.rootgrid
    pm = sum(1 << a for a in range(3) if rg.periodic[a])
    fin, fout = tmp / "in.bin", tmp / "out.bin"
    with open(fin, "wb") as fp:
        fp.write(np.array([rg.nx, rg.ny, rg.nz, pm, n, vc, tree.num_leaves, mode, n_pre,
                           max_iter], np.int32).tobytes())
        fp.write(np.array([omega, eps], np.float64).tobytes())
        fp.write(np.ascontiguousarray(tree.pedigrees, np.uint64).tobytes())
        for a in list(fields) + [b, x]:
            fp.write(np.ascontiguousarray(a, np.float64).tobytes())
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([str(BIN), str(fin), str(fout)], check=True, env=env, timeout=300)
    raw = fout.read_bytes()
    count = int(np.frombuffer(raw, np.int32, 1, 0)[0])
    res = float(np.frombuffer(raw, np.float64, 1, 4)[0])
    xr = np.frombuffer(raw, np.float64, x.size, 12).reshape(x.shape)
    return count, res, xr


@pytest.fixture
def one_thread():
    before = po.num_threads()
    po.set_threads(1)
    yield
    po.set_threads(before)


@pytest.mark.parametrize("n_pre,max_iter,eps", [(2, 300, 1e-9), (1, 300, 1e-9), (2, 7, 1e-30)])
def test_bicgstab_matches_reference_ils3d(tmp_path, one_thread, n_pre, max_iter, eps):
    n, vc, omega = 8, 1, 0.8
    tree, m, fields, b, bct, bcv = _system(n, vc)
    x0 = np.zeros(m.shape)
    count, res, xr = _run_reference(tree, n, vc, fields, b, x0, 1, n_pre, max_iter, omega, eps,
                                    tmp_path)
    x = x0.copy()
    it, res_o = m.bicgstab(x, b, omega, n_pre, max_iter, eps, bct, bcv, 0, fields=fields)
    assert count > 0
    assert it == (max_iter if count == max_iter + 1 else count)
    assert res_o == res
    inner = (slice(None), slice(vc, -vc), slice(vc, -vc), slice(vc, -vc))
    assert np.array_equal(x[inner], xr[inner])


def test_jacobi_matches_reference_ils3d(tmp_path, one_thread):
    n, vc, omega = 8, 1, 0.9
    tree, m, fields, b, bct, bcv = _system(n, vc, seed=5)
    x0 = np.zeros(m.shape)
    count, res, xr = _run_reference(tree, n, vc, fields, b, x0, 0, 0, 40, omega, 1e-30,
                                    tmp_path)
    x = x0.copy()
    it, res_o = m.jacobi_solve(x, b, omega, 40, 1e-30, bct, bcv, 0, fields=fields)
    assert count == 41 and it == 40  # the limit: ILS3D's loop variable ends at countMax + 1
    assert res_o == res
    inner = (slice(None), slice(vc, -vc), slice(vc, -vc), slice(vc, -vc))
    assert np.array_equal(x[inner], xr[inner])
