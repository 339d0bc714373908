"""Served solves: a stream of independent Poisson problems, each solved to a
relative residual target by the mixed-precision BiCGSTAB, admitted against a
device-memory budget as memory frees up, with the iterations of the requests
on the device batched together.

The reference solves one problem per BlockManager in one process
(SolverTest: ILS3D::BiCGSTAB, ILS3D.h:663-844).  Here (`BatchServer`) the
requests waiting when a worker frees up are packed into one block set (their
blocks concatenated, bcmtools_gb300.batch.Batch), each request a segment of
it (bcmg_set_segments): one mixed-precision call then advances every request
of the batch with every launch, each with its own scalars, refinement history
and convergence test, so its result is the one it gets solved alone.  Batches
take requests of one block edge and similar size (within `size_ratio` of the
oldest waiting request, which is always admitted first), and several workers
run batches concurrently on their own streams as the device-byte budget
allows: requests that arrive while others are on the device are admitted as
soon as a worker and memory free up.  `Server` is the earlier design -- one
context per request, concurrency from stream overlap alone -- and
`one_at_a_time` the plain loop the served throughput is compared with.
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

    _spec: Optional[tuple] = field(default=None, repr=False, compare=False)

    def mesh_spec(self):
        """(RootGrid, Divider) of the request's mesh: refined to `level`
        around seeded points, the balls' radius bisected until the leaf count
        is near target_cells / n^3 (2:1 balanced); the coarsest level is 2 for
        meshes of 64 blocks or more, else as coarse as the target needs (one
        root block is 4096 cells at n = 16).  The bisection is the stream
        generator's (host trees, once per request); the server builds the
        mesh from the spec on the device."""
        if self._spec is None:
            rng = np.random.default_rng(self.seed)
            target = max(1.0, self.target_cells / self.n ** 3)
            min_level = 2 if target >= 64 else (1 if target >= 8 else 0)
            level = max(self.level, min_level)
            pts = rng.uniform(0.0, 1.0, size=(int(rng.integers(1, 5)), 3))
            lo, hi = 1e-3, 1.0
            div = None
            for _ in range(24):
                r = float(np.sqrt(lo * hi))
                div = Divider.balls(pts, r, level, min_level=min_level)
                nl = Octree.build(RootGrid(1, 1, 1), div, "Z").num_leaves
                if nl < target:
                    lo = r
                else:
                    hi = r
                if abs(nl - target) < 0.2 * target:
                    break
            self._spec = (RootGrid(1, 1, 1), div)
        return self._spec

    def build(self) -> Octree:
        """The request's mesh as a host octree (mesh_spec)."""
        rg, div = self.mesh_spec()
        return Octree.build(rg, div, "Z")

    def device_bytes(self, nb: int) -> int:
        return int(nb * (self.n + 2) ** 3 * BYTES_PER_CELL)


def poisson_stream(count: int, rate: float, seed: int, cells=(1e4, 1e8), sizes=(16, 32),
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
    setup_s: float = 0.0   # set-up time: mesh built, registered, fields made (its share)
    batch: int = 1         # requests solved together with it (itself included)

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


def solve_alone(req: Request, device: int = 0, keep: bool = False,
                tree: Optional[Octree] = None):
    """One request in its own context: Dirichlet 0 on the outer faces,
    seeded uniform [-1,1] right-hand side, mixed-precision BiCGSTAB (Jacobi
    preconditioner, two passes at omega 0.8) to req.eps.  Returns (info,
    blocks, cells, x or None)."""
    return _solve_one(req, device, keep, tree, True, solve_alone)


def solve_plain(req: Request, device: int = 0, keep: bool = False,
                tree: Optional[Octree] = None):
    """The plain path for one request: the same system solved by the FP64
    BiCGSTAB (ILS3D::BiCGSTAB, ILS3D.h:663-844, in the reference's double
    precision: vectors, stencil and scalars in FP64) to req.eps, with the
    same preconditioner.  Returns (info, blocks, cells, x or None)."""
    return _solve_one(req, device, keep, tree, False, solve_plain)


def _solve_one(req: Request, device: int, keep: bool, tree: Optional[Octree], mixed: bool,
               owner: Callable):
    t0 = time.perf_counter()
    bm = BlockManager(device)
    try:
        n = req.n
        if tree is not None:
            ld, nid, sf, outer = tree.neighbors()
            bm.register_blocks(ld, nid, sf, n)
        else:  # the mesh made on the device from the request's spec
            tree = bm.build_mesh(*req.mesh_spec(), n)
            outer = bm.outer
        t = np.where(outer != 0, BC_DIRICHLET, 0).astype(np.int32)
        bm.set_boundary(t, np.zeros(t.shape), DIRICHLET_SOR)
        op = bm.op_const(laplace_coef(tree.cell_sizes(n)))
        x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
        b.fill(0.0)
        b.fill_random(req.seed)
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        owner.last_setup = time.perf_counter() - t0
        # omega 0.8: two undamped Jacobi passes annihilate the checkerboard
        # mode of a uniform grid (their polynomial l(2 - l) vanishes at l = 2),
        # so the right preconditioner is singular there and BiCGSTAB blows up
        # on flat meshes -- the reference's ILS3D::BiCGSTAB does the same
        if mixed:
            info = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=400,
                                     eps_inner=1e-4, max_outer=30, eps=req.eps)
        else:
            info = bm.bicgstab(op, x, b, omega=0.8, n_pre=2, max_iter=20000, eps=req.eps)
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


@dataclass
class _Mesh:
    tree: Octree
    n: int
    vc: int = 1


def solve_batch(reqs: Sequence[Request], device: int = 0, keep: bool = False,
                trees: Optional[Sequence[Octree]] = None, stream=None):
    """Requests of one block edge solved together: their meshes concatenated
    into one block set, each request a segment, one mixed-precision BiCGSTAB
    call (Jacobi preconditioner, two passes at omega 0.8) to each request's
    eps (the batch's smallest).  Returns ([(info, blocks, cells, x or None)],
    seconds of set-up: the meshes built on the device, registration, fields)."""
    from .batch import Batch
    t0 = time.perf_counter()
    n = reqs[0].n
    if trees is not None:
        trees = list(trees)
        batch = Batch([_Mesh(t, n) for t in trees], device)
    else:  # the meshes made on the device from the requests' specs, in one call
        batch = Batch.from_dividers([r.mesh_spec() for r in reqs], n, 1, device)
        trees = [w.tree for w in batch.workloads]
    try:
        batch.set_dirichlet(0.0)
        op = batch.laplace_op()
        bm = batch.bm
        x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
        batch.fill_rhs(b, [r.seed for r in reqs])
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        batch.set_segments()
        setup = time.perf_counter() - t0
        infos = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=400, eps_inner=1e-4,
                                  max_outer=30, eps=min(r.eps for r in reqs), stream=stream)
        if not isinstance(infos, list):
            infos = [infos]
        xh = x.download() if keep else None
        out = []
        for k, t in enumerate(trees):
            xk = batch.instance(xh, k).copy() if keep else None
            out.append((infos[k], t.num_leaves, t.num_leaves * n ** 3, xk))
        return out, setup
    finally:
        batch.bm.close()


class BatchServer:
    """Continuous batching.  A worker that is free takes the oldest waiting
    request that has arrived and, with it, the other arrived requests of the
    same block edge whose size is within `size_ratio` of it, while the
    batch's device bytes fit what the budget has left (a request larger than
    the whole budget goes alone) and the batch holds at most
    `max_batch_cells` cells and `max_batch` requests; it solves them as one
    batch (solve_batch) on its own stream.  `workers` batches run at once."""

    def __init__(self, device: int = 0, budget_bytes: float = 150e9, workers: int = 4,
                 size_ratio: float = 4.0, max_batch_cells: float = 2e8, max_batch: int = 256,
                 solver: Optional[Callable] = None,
                 clock: Callable[[], float] = time.perf_counter,
                 sleep: Callable[[float], None] = time.sleep):
        self.device, self.budget, self.workers = device, float(budget_bytes), workers
        self.size_ratio, self.max_cells, self.max_batch = size_ratio, max_batch_cells, max_batch
        self.solver = solver or solve_batch
        self.clock, self.sleep = clock, sleep

    def _cost(self, r: Request) -> float:
        return float(r.target_cells) * (1 + 2.0 / r.n) ** 3 * BYTES_PER_CELL

    def run(self, requests: Sequence[Request], keep: bool = False) -> List[Result]:
        waiting = sorted(requests, key=lambda r: r.arrival)
        lock = threading.Condition()
        state = {"inflight": 0.0, "running": 0, "batches": 0}
        results: List[Result] = []
        errors = []
        t0 = self.clock()

        def take(now: float):
            """The next batch among the requests arrived by `now` (lock held)."""
            arrived = [r for r in waiting if r.arrival <= now]
            if not arrived:
                return None
            head = arrived[0]
            room = self.budget - state["inflight"]
            if self._cost(head) > room and state["running"] > 0:
                return None
            batch, cost, cells = [head], self._cost(head), head.target_cells
            for r in arrived[1:]:
                if len(batch) >= self.max_batch:
                    break
                if r.n != head.n:
                    continue
                ratio = r.target_cells / head.target_cells
                if not (1.0 / self.size_ratio <= ratio <= self.size_ratio):
                    continue
                c = self._cost(r)
                if cost + c > room or cells + r.target_cells > self.max_cells:
                    continue
                batch.append(r)
                cost += c
                cells += r.target_cells
            for r in batch:
                waiting.remove(r)
            state["inflight"] += cost
            state["running"] += 1
            state["batches"] += 1
            return batch, cost

        def worker():
            while True:
                with lock:
                    while True:
                        if not waiting:
                            return
                        now = self.clock() - t0
                        got = take(now)
                        if got is not None:
                            break
                        nxt = min(r.arrival for r in waiting)
                        lock.wait(timeout=max(1e-4, nxt - now) if nxt > now else 0.05)
                batch, cost = got
                start = self.clock() - t0
                try:
                    out, setup = self.solver(batch, self.device, keep)
                    fin = self.clock() - t0
                    cells_all = sum(o[2] for o in out)
                    res = [Result(r.rid, r.arrival, start, fin, o[1], o[2], o[0].iterations,
                                  o[0].refinements, o[0].true_residual, o[0].status, o[3],
                                  setup * o[2] / max(1, cells_all), len(batch))
                           for r, o in zip(batch, out)]
                except Exception as e:  # recorded, the stream goes on
                    errors.append(([r.rid for r in batch], repr(e)))
                    fin = self.clock() - t0
                    res = [Result(r.rid, r.arrival, start, fin, 0, 0, 0, 0, float("nan"), -1,
                                  None, 0.0, len(batch)) for r in batch]
                with lock:
                    results.extend(res)
                    state["inflight"] -= cost
                    state["running"] -= 1
                    lock.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.workers)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        self.errors = errors
        self.batches = state["batches"]
        return sorted(results, key=lambda r: r.rid)


def one_at_a_time(requests: Sequence[Request], device: int = 0, keep: bool = False,
                  solver: Callable = solve_alone, clock=time.perf_counter,
                  sleep=time.sleep) -> List[Result]:
    """The plain loop: requests in arrival order, one at a time."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    out = []
    t0 = clock()
    for r in reqs:
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            sleep(wait)
        start = clock() - t0
        info, nb, cells, xh = solver(r, device, keep, None)
        out.append(Result(r.rid, r.arrival, start, clock() - t0, nb, cells, info.iterations,
                          info.refinements, info.true_residual, info.status, xh,
                          getattr(solver, "last_setup", 0.0)))
    return out


def summary(results: Sequence[Result]) -> dict:
    lat = np.array([r.latency for r in results])
    span = max(r.finish for r in results) - min(r.arrival for r in results)
    busy = sum(r.finish - r.start for r in results)
    return {"requests": len(results), "solves_per_s": len(results) / span,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": span, "cells": int(sum(r.cells for r in results)),
            "max_residual": float(max(r.residual for r in results)),
            "failed": int(sum(1 for r in results if r.status != 0)),
            "host_setup_s": float(sum(r.setup_s for r in results)),
            # set-up against the solve time of the batches (each batch once)
            "setup_share": float(sum(r.setup_s for r in results) /
                                 max(1e-12, sum((r.finish - r.start) / max(1, r.batch)
                                                for r in results))),
            "mean_batch": float(np.mean([r.batch for r in results])),
            "busy_s": float(busy)}
