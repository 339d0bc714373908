"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: meshes come from the octree builder and right
hand sides from numpy's seeded generators.

  plain_poisson      512 uniform blocks of 16^3, vc=1 (root 1^3, flat level 3)
  two_level_sphere   root 4^3 grid over [0,1]^3 refined to level 3 where blocks
                     meet the sphere |x - c| = 0.3, c = (0.5,0.5,0.5); 2:1
                     balanced; 16^3 cells, vc=2
  points_level5      root 1^3 refined to level 5 around 16 seeded points
                     (radius 0.05); 2:1 balanced; 32^3 cells, vc=1
  random_instance    one instance of the batched / served mixes
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .blockmanager import BC_DIRICHLET
from .mesh import Divider, Octree, RootGrid


@dataclass
class Workload:
    name: str
    tree: Octree
    n: int
    vc: int

    @property
    def nb(self) -> int:
        return self.tree.num_leaves

    @property
    def cells(self) -> int:
        return self.nb * self.n ** 3

    def neighbors(self):
        return self.tree.neighbors()

    def dirichlet(self, value: float = 0.0):
        """Dirichlet on every outer face (sor2 BoundaryConditionSetter.h:43-49)."""
        _, _, _, outer = self.tree.neighbors()
        t = np.where(outer != 0, BC_DIRICHLET, 0).astype(np.int32)
        v = np.where(outer != 0, value, 0.0)
        return t, v

    def cell_centres(self):
        """(nb, n, n, n, 3) cell-centre coordinates, z-major like the bricks."""
        n = self.n
        h = self.tree.block_sizes / n
        o = self.tree.origins
        idx = np.arange(n) + 0.5
        x = o[:, 0, None] + idx[None, :] * h[:, None]
        y = o[:, 1, None] + idx[None, :] * h[:, None]
        z = o[:, 2, None] + idx[None, :] * h[:, None]
        return x, y, z


def plain_poisson(n: int = 16, vc: int = 1, level: int = 3) -> Workload:
    rg = RootGrid(1, 1, 1)
    d = Divider.flat(level)
    return Workload("plain_poisson", Octree.build(rg, d, "Z"), n, vc)


def two_level_sphere(n: int = 16, vc: int = 2, level: int = 3, ordering: str = "Z") -> Workload:
    rg = RootGrid(4, 4, 4, root_length=0.25)
    d = Divider.sphere_surface((0.5, 0.5, 0.5), 0.3, level)
    return Workload("two_level_sphere", Octree.build(rg, d, ordering), n, vc)


def points_level5(n: int = 32, vc: int = 1, level: int = 5, seed: int = 3,
                  npoints: int = 16, radius: float = 0.05) -> Workload:
    pts = np.random.default_rng(seed).uniform(0.0, 1.0, size=(npoints, 3))
    rg = RootGrid(1, 1, 1)
    d = Divider.balls(pts, radius, level)
    return Workload("points_level5", Octree.build(rg, d, "Z"), n, vc)


def random_instance(seed: int, min_blocks: int = 64, max_blocks: int = 4096,
                    sizes=(8, 16, 32)) -> Workload:
    """Batched-mix instance: block count log-uniform in [min, max] (reached
    by refining around seeded points), cell size drawn from `sizes`."""
    rng = np.random.default_rng(seed)
    target = float(np.exp(rng.uniform(np.log(min_blocks), np.log(max_blocks))))
    n = int(rng.choice(sizes))
    level = max(2, int(np.ceil(np.log(target) / np.log(8))) + 1)
    pts = rng.uniform(0.0, 1.0, size=(int(rng.integers(1, 9)), 3))
    lo, hi = 1e-3, 1.0
    tree = None
    for _ in range(30):
        r = np.sqrt(lo * hi)
        t = Octree.build(RootGrid(1, 1, 1), Divider.balls(pts, r, level, min_level=2), "Z")
        tree = t
        if t.num_leaves < target:
            lo = r
        else:
            hi = r
        if abs(t.num_leaves - target) < 0.15 * target:
            break
    return Workload(f"instance{seed}", tree, n, 1)


def rhs_uniform(w: Workload, seed: int, dtype=np.float32, zero_mean: bool = True) -> np.ndarray:
    """Interior RHS uniform[-1,1] (mean removed) in the brick layout."""
    rng = np.random.default_rng(seed)
    n, vc = w.n, w.vc
    b = np.zeros((w.nb, n + 2 * vc, n + 2 * vc, n + 2 * vc), dtype)
    v = rng.uniform(-1.0, 1.0, size=(w.nb, n, n, n))
    if zero_mean:
        v -= v.mean()
    b[:, vc:-vc, vc:-vc, vc:-vc] = v
    return b


def rhs_gaussian(w: Workload, seed: int, dtype=np.float32, sigma: float = 0.1,
                 noise: float = 0.01, centre=(0.5, 0.5, 0.5)) -> np.ndarray:
    """Gaussian blob (sigma) at `centre` plus uniform[-noise, noise]."""
    rng = np.random.default_rng(seed)
    n, vc = w.n, w.vc
    x, y, z = w.cell_centres()
    r2 = ((z[:, :, None, None] - centre[2]) ** 2 + (y[:, None, :, None] - centre[1]) ** 2
          + (x[:, None, None, :] - centre[0]) ** 2)
    v = np.exp(-r2 / (2 * sigma * sigma)) + rng.uniform(-noise, noise, size=r2.shape)
    b = np.zeros((w.nb, n + 2 * vc, n + 2 * vc, n + 2 * vc), dtype)
    b[:, vc:-vc, vc:-vc, vc:-vc] = v
    return b


def _splitmix64(z: np.ndarray) -> np.ndarray:
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def rhs_fill_random(w: Workload, seed: int, dtype=np.float64, lo: float = -1.0,
                    hi: float = 1.0) -> np.ndarray:
    """Host copy of Scalar3D.fill_random(seed, lo, hi) on every block
    (bcmg_field_fill_random): the value of interior cell c of block l is
    lo + (hi - lo) u with u the top 53 bits of splitmix64(seed * 0x100000001b3
    ^ splitmix64(l * n^3 + c)), ghosts zero.  For the default [-1, 1) the
    product (hi - lo) u is exact, so the device's contraction of the update
    into one multiply-add cannot change the value."""
    n, vc = w.n, w.vc
    cells = n ** 3
    out = np.zeros((w.nb, n + 2 * vc, n + 2 * vc, n + 2 * vc), dtype)
    s = np.uint64(seed) * np.uint64(0x100000001B3)
    c = np.arange(cells, dtype=np.uint64)
    with np.errstate(over="ignore"):
        for l in range(w.nb):
            h = _splitmix64(s ^ _splitmix64(np.uint64(l) * np.uint64(cells) + c))
            u = (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
            out[l, vc:-vc, vc:-vc, vc:-vc] = (lo + (hi - lo) * u).reshape(n, n, n)
    return out
