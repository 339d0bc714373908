"""Served solves: a stream of independent Poisson problems, each solved to a
relative residual target by the mixed-precision BiCGSTAB, admitted against a
device-memory budget and run concurrently.

The reference solves one problem per BlockManager in one process
(SolverTest: ILS3D::BiCGSTAB, ILS3D.h:663-844).  Here every request gets its
own context (block set, face table, fields, CUDA stream) so requests never
share device state and a request's result does not depend on what runs beside
it; worker threads drive the contexts concurrently (the library's calls
release the interpreter lock), and admission is first-come first-served
within the memory budget.  `solve_alone` is the one-at-a-time path the
served throughput is compared with.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from .blockmanager import BC_DIRICHLET, DIRICHLET_SOR, BlockManager, laplace_coef
from .mesh import Divider, Octree, RootGrid

# device bytes per padded brick cell of one request: x, b (FP64) plus the
# FP64 residual / correction and the FP32 BiCGSTAB vectors of the mixed solver
BYTES_PER_CELL = 2 * 8 + 3 * 8 + 10 * 4


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the stream starts
    n: int                  # block edge
    level: int              # maximum refinement level
    target_cells: int
    seed: int
    eps: float = 1e-8

    def build(self) -> Octree:
        """Octree refined to `level` around seeded points, its radius bisected
        until the leaf count is near target_cells / n^3 (2:1 balanced)."""
        rng = np.random.default_rng(self.seed)
        target = max(64.0, self.target_cells / self.n ** 3)
        pts = rng.uniform(0.0, 1.0, size=(int(rng.integers(1, 5)), 3))
        lo, hi = 1e-3, 1.0
        tree = None
        for _ in range(24):
            r = float(np.sqrt(lo * hi))
            tree = Octree.build(RootGrid(1, 1, 1), Divider.balls(pts, r, self.level, min_level=2),
                                "Z")
            if tree.num_leaves < target:
                lo = r
            else:
                hi = r
            if abs(tree.num_leaves - target) < 0.2 * target:
                break
        return tree

    def device_bytes(self, nb: int) -> int:
        return int(nb * (self.n + 2) ** 3 * BYTES_PER_CELL)


def poisson_stream(count: int, rate: float, seed: int, cells=(2.6e5, 8e6), sizes=(16, 32),
                   levels=(2, 6), eps=1e-8) -> List[Request]:
    """`count` requests with Poisson arrivals at `rate` per second; cells
    log-uniform in `cells`; block edge from `sizes` (the larger only when it
    still gives at least 64 blocks); maximum level uniform in `levels`."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += float(rng.exponential(1.0 / rate))
        c = float(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1]))))
        fits = [n for n in sizes if c / n ** 3 >= 64]
        n = int(rng.choice(fits if fits else [min(sizes)]))
        lv = int(rng.integers(levels[0], levels[1] + 1))
        out.append(Request(k, t, n, lv, int(c), int(rng.integers(1 << 31)), eps))
    return out


@dataclass
class Result:
    rid: int
    arrival: float
    start: float
    finish: float
    blocks: int
    cells: int
    iterations: int
    refinements: int
    residual: float
    status: int
    x: Optional[np.ndarray] = field(default=None, repr=False)

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


def solve_alone(req: Request, device: int = 0, keep: bool = False,
                tree: Optional[Octree] = None):
    """One request in its own context: Dirichlet 0 on the outer faces,
    seeded uniform [-1,1] right-hand side, mixed-precision BiCGSTAB (Jacobi
    preconditioner, two passes at omega 0.8) to req.eps.  Returns (info,
    blocks, cells, x or None)."""
    tree = tree if tree is not None else req.build()
    bm = BlockManager(device)
    try:
        n = req.n
        ld, nid, sf, outer = tree.neighbors()
        bm.register_blocks(ld, nid, sf, n)
        t = np.where(outer != 0, BC_DIRICHLET, 0).astype(np.int32)
        bm.set_boundary(t, np.zeros(t.shape), DIRICHLET_SOR)
        op = bm.op_const(laplace_coef(tree.cell_sizes(n)))
        x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
        b.fill(0.0)
        b.fill_random(req.seed)
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        # omega 0.8: two undamped Jacobi passes annihilate the checkerboard
        # mode of a uniform grid (their polynomial l(2 - l) vanishes at l = 2),
        # so the right preconditioner is singular there and BiCGSTAB blows up
        # on flat meshes -- the reference's ILS3D::BiCGSTAB does the same
        info = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=400, eps_inner=1e-4,
                                 max_outer=30, eps=req.eps)
        xh = x.download() if keep else None
        return info, tree.num_leaves, tree.num_leaves * n ** 3, xh
    finally:
        bm.close()


class Server:
    """Admits requests in arrival order while the sum of their device-byte
    estimates stays within `budget_bytes`; `workers` threads solve the
    admitted ones concurrently, each in its own context.  A request larger
    than the whole budget is admitted alone."""

    def __init__(self, device: int = 0, budget_bytes: float = 150e9, workers: int = 8,
                 solver: Callable = solve_alone, clock: Callable[[], float] = time.perf_counter,
                 sleep: Callable[[float], None] = time.sleep):
        self.device, self.budget, self.workers = device, float(budget_bytes), workers
        self.solver, self.clock, self.sleep = solver, clock, sleep

    def run(self, requests: Sequence[Request], keep: bool = False) -> List[Result]:
        reqs = sorted(requests, key=lambda r: r.arrival)
        trees = {r.rid: r.build() for r in reqs}  # host meshes ahead of time
        cost = {r.rid: r.device_bytes(trees[r.rid].num_leaves) for r in reqs}
        lock = threading.Condition()
        state = {"next": 0, "inflight": 0.0, "running": 0}
        results: List[Result] = []
        t0 = self.clock()
        errors = []

        def worker():
            while True:
                with lock:
                    while True:
                        k = state["next"]
                        if k >= len(reqs):
                            return
                        r = reqs[k]
                        c = cost[r.rid]
                        fits = state["inflight"] + c <= self.budget or state["running"] == 0
                        if fits:
                            state["next"] += 1
                            state["inflight"] += c
                            state["running"] += 1
                            break
                        lock.wait()
                wait = r.arrival - (self.clock() - t0)
                if wait > 0:
                    self.sleep(wait)
                start = self.clock() - t0
                try:
                    info, nb, cells, xh = self.solver(r, self.device, keep, trees[r.rid])
                    res = Result(r.rid, r.arrival, start, self.clock() - t0, nb, cells,
                                 info.iterations, info.refinements, info.true_residual,
                                 info.status, xh)
                except Exception as e:  # recorded, the stream goes on
                    errors.append((r.rid, repr(e)))
                    res = Result(r.rid, r.arrival, start, self.clock() - t0, 0, 0, 0, 0,
                                 float("nan"), -1, None)
                with lock:
                    results.append(res)
                    state["inflight"] -= c
                    state["running"] -= 1
                    lock.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.workers)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        self.errors = errors
        return sorted(results, key=lambda r: r.rid)


def one_at_a_time(requests: Sequence[Request], device: int = 0, keep: bool = False,
                  solver: Callable = solve_alone, clock=time.perf_counter,
                  sleep=time.sleep) -> List[Result]:
    """The plain loop: requests in arrival order, one at a time."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    trees = {r.rid: r.build() for r in reqs}
    out = []
    t0 = clock()
    for r in reqs:
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            sleep(wait)
        start = clock() - t0
        info, nb, cells, xh = solver(r, device, keep, trees[r.rid])
        out.append(Result(r.rid, r.arrival, start, clock() - t0, nb, cells, info.iterations,
                          info.refinements, info.true_residual, info.status, xh))
    return out


def summary(results: Sequence[Result]) -> dict:
    lat = np.array([r.latency for r in results])
    span = max(r.finish for r in results) - min(r.arrival for r in results)
    return {"requests": len(results), "solves_per_s": len(results) / span,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": span, "cells": int(sum(r.cells for r in results)),
            "max_residual": float(max(r.residual for r in results)),
            "failed": int(sum(1 for r in results if r.status != 0))}
