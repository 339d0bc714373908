"""Makes tests/golden/c3_points_level5_fp64.npz: the FP64 CPU oracle's
BiCGSTAB solution of the mixed-precision benchmark's system.

System (the mixed_bicgstab workload of bench.py): the level-5 octree around
16 seeded points (seed 3, radius 0.05, 2:1 balanced), 32^3 cells per block,
vc = 1, 7-point Laplacian with per-block constant coefficients, Dirichlet 0
ghosts (2v - f form), right-hand side Scalar3D.fill_random(3) (uniform
[-1, 1) on every interior cell), x = 0.  Solved by the oracle's restatement
of ILS3D::BiCGSTAB (examples/SolverTest/ILS3D.h:663-844) in FP64 with the
Jacobi preconditioner (2 passes, omega 0.8) to |r|^2/|b|^2 <= (1e-12)^2, on
all host cores (oracle/bcm_oracle.c, OpenMP).

Stored: the iteration count and final residual, the L2 norm and maximum of
the solution, per-block sums of squares and maxima of |x| over the interior,
and eight whole blocks spread over the mesh (the full solution is 0.8 GB).
The GPU's mixed-precision solve is checked against these (bench.py
--workload mixed_bicgstab reports the error; the GPU tests compare the
right-hand side generator).  Takes about half an hour on 8 cores.

    python tests/golden/make_c3_fixture.py
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

OMEGA, N_PRE, EPS, MAX_ITER, SEED = 0.8, 2, 1e-12, 4000, 3


def main() -> int:
    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    from oracle import pyoracle as po
    w = W.points_level5()
    ld, nid, sf, _ = w.neighbors()
    bct, bcv = w.dirichlet(0.0)
    cc = bg.laplace_coef(w.tree.cell_sizes(w.n))
    b = W.rhs_fill_random(w, SEED, np.float64)
    m = po.OracleMesh(ld, nid, sf, w.n, w.vc)
    x = np.zeros(m.shape, np.float64)
    m.vc_update(x)
    m.dirichlet(x, bct, bcv, 0)
    t0 = time.perf_counter()
    it, res = m.bicgstab(x, b, OMEGA, N_PRE, MAX_ITER, EPS, bct, bcv, 0, cc=cc)
    secs = time.perf_counter() - t0
    inner = x[:, 1:-1, 1:-1, 1:-1]
    sumsq = (inner * inner).sum(axis=(1, 2, 3))
    bmax = np.abs(inner).max(axis=(1, 2, 3))
    picks = np.unique(np.linspace(0, w.nb - 1, 8).round().astype(np.int64))
    np.savez_compressed(
        HERE / "c3_points_level5_fp64.npz", nb=w.nb, n=w.n, vc=w.vc, omega=OMEGA, n_pre=N_PRE,
        eps=EPS, seed=SEED, iterations=it, residual=res, norm=float(np.sqrt(sumsq.sum())),
        xmax=float(bmax.max()), block_sumsq=sumsq, block_max=bmax, sample_ids=picks,
        sample_blocks=inner[picks], pedigrees=w.tree.pedigrees, cpu_seconds=secs,
        cpu_threads=po.num_threads())
    print(f"{w.nb} blocks, {it} iterations, residual {res:.3e}, {secs:.0f} s on "
          f"{po.num_threads()} threads")
    return 0


if __name__ == "__main__":
    sys.exit(main())
