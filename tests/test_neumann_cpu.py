"""CPU: Neumann ghosts of the oracle (SolverTest/bcx.f90:198-376) against a
direct restatement -- first layer interior -/+ xc in the field's type, second
layer interior -/+ 2 xc evaluated in double."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import small_octree


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("vc", [1, 2])
def test_oracle_neumann_ghosts(dt, vc):
    n = 8
    tree = small_octree(periodic=(False, False, False), level=1, radius=0.3)
    ld, nid, sf, outer = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    nb = ld.shape[0]
    rng = np.random.default_rng(3)
    a = rng.uniform(-1, 1, size=(nb, n + 2 * vc, n + 2 * vc, n + 2 * vc)).astype(dt)
    bct = np.where(outer != 0, 2, 0).astype(np.int32)  # Neumann on every outer face
    bcv = rng.uniform(-0.1, 0.1, size=(nb, 6))
    got = a.copy()
    m.dirichlet(got, bct, bcv, 0)
    want = a.copy()
    v = vc
    for b in range(nb):
        for f in range(6):
            if bct[b, f] != 2:
                continue
            xc = dt(bcv[b, f])
            ax, minus = f // 2, f % 2 == 0
            sl = [slice(v, v + n)] * 3  # (z, y, x) interior
            axis = 2 - ax  # array axis of face axis ax
            idx = list(sl)
            idx[axis] = v if minus else v + n - 1
            interior = want[b][tuple(idx)]
            g1 = list(sl)
            g1[axis] = v - 1 if minus else v + n
            want[b][tuple(g1)] = (interior - xc) if minus else (interior + xc)
            if vc >= 2:
                g2 = list(sl)
                g2[axis] = v - 2 if minus else v + n + 1
                sgn = -1.0 if minus else 1.0
                want[b][tuple(g2)] = (interior.astype(np.float64)
                                      + sgn * (np.float64(xc) * 2.0)).astype(dt)
    assert np.array_equal(got, want)
