"""CPU: boundary folding of a coefficient-brick operator in the oracle
(SolverTest bca.f90:12-394, LocalScalar3D.h:260-285) against a direct numpy
restatement -- per cell the x-, x+, y-, y+, z-, z+ faces in turn; Dirichlet
Ap -= A_nb, b = b - 2 (A_nb xc) with the product in the field's type and the
rest in double; Neumann Ap += A_nb, b +/- A_nb xc in the field's type; the
folded coefficient set to 0; faces with a neighbour left alone."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import small_octree


def fold_numpy(A, b, bct, bcv, nid, n, vc):
    A = [a.copy() for a in A]
    b = b.copy()
    nb = b.shape[0]
    dt = b.dtype.type
    for blk in range(nb):
        for f in range(6):
            t = bct[blk, f]
            if t not in (1, 2) or (nid[blk, f] >= 0).any():
                continue
            ax, minus = f // 2, f % 2 == 0
            axis = 2 - ax  # array axis (z, y, x) of face axis ax
            idx = [slice(vc, vc + n)] * 3
            idx[axis] = vc if minus else vc + n - 1
            idx = (blk,) + tuple(idx)
            xc = dt(bcv[blk, f])
            a = A[1 + f][idx].copy()
            p = (a * xc).astype(b.dtype)
            if t == 1:
                A[0][idx] = A[0][idx] - a
                b[idx] = (b[idx].astype(np.float64) - p.astype(np.float64) * 2.0).astype(b.dtype)
            else:
                A[0][idx] = A[0][idx] + a
                b[idx] = (b[idx] + p) if minus else (b[idx] - p)
            A[1 + f][idx] = 0
    return A, b


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 4])
def test_oracle_fold_matches_restatement(dt, n):
    vc = 1
    tree = small_octree(periodic=(False, True, False), level=1, radius=0.3)
    ld, nid, sf, outer = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    nb = ld.shape[0]
    rng = np.random.default_rng(21)
    shape = (nb, n + 2 * vc, n + 2 * vc, n + 2 * vc)
    A = [rng.uniform(-1, 1, size=shape).astype(dt) for _ in range(7)]
    b = rng.uniform(-1, 1, size=shape).astype(dt)
    # Dirichlet on x, Neumann on z, a Dirichlet type on the periodic y faces
    # (they have neighbours, so nothing folds there)
    bct = np.zeros((nb, 6), np.int32)
    bct[:, 0:2] = 1
    bct[:, 2:4] = 1
    bct[:, 4:6] = 2
    bcv = rng.uniform(-0.5, 0.5, size=(nb, 6))
    want_A, want_b = fold_numpy(A, b, bct, bcv, nid.reshape(nb, 6, 4), n, vc)
    got_A = [a.copy() for a in A]
    got_b = b.copy()
    m.fold(got_A, got_b, bct, bcv)
    for k in range(7):
        assert np.array_equal(got_A[k], want_A[k]), k
    assert np.array_equal(got_b, want_b)
    assert not np.array_equal(got_b, b)  # something folded
