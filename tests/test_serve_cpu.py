"""CPU: the served-stream scheduler (bcmtools_gb300.serve) with a stand-in
solver -- arrivals, first-come-first-served admission within the memory
budget, concurrency, and the one-at-a-time loop.  No device work."""
import threading
import time
from types import SimpleNamespace

import numpy as np

from bcmtools_gb300 import serve


def fake_solver(record, dt=0.02):
    lock = threading.Lock()

    def solve(req, device, keep, tree):
        tree = tree if tree is not None else req.build()
        nb = tree.num_leaves
        with lock:
            record["inflight"] += req.device_bytes(nb)
            record["peak"] = max(record["peak"], record["inflight"])
            record["running"] += 1
            record["max_running"] = max(record["max_running"], record["running"])
            record["order"].append(req.rid)
        time.sleep(dt)
        with lock:
            record["inflight"] -= req.device_bytes(nb)
            record["running"] -= 1
        info = SimpleNamespace(iterations=1, refinements=0, true_residual=0.0, status=0)
        return info, nb, nb * req.n ** 3, None

    return solve


def small_stream(count=12, rate=400.0):
    return serve.poisson_stream(count, rate, seed=5, cells=(3e4, 3e5), sizes=(8, 16),
                                levels=(2, 3))


def test_poisson_stream_is_seeded_and_ordered():
    a, b = small_stream(), small_stream()
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    gaps = np.diff([0.0] + [r.arrival for r in serve.poisson_stream(2000, 200.0, seed=5)])
    assert abs(gaps.mean() - 1 / 200.0) < 0.15 / 200.0  # exponential gaps at rate 200/s


def test_server_respects_budget_and_order():
    reqs = small_stream()
    trees = {r.rid: r.build() for r in reqs}
    costs = sorted(r.device_bytes(trees[r.rid].num_leaves) for r in reqs)
    budget = costs[-1] + costs[-2]  # room for two of the largest at once
    rec = {"inflight": 0, "peak": 0, "running": 0, "max_running": 0, "order": []}
    res = serve.Server(budget_bytes=budget, workers=6, solver=fake_solver(rec)).run(reqs)
    assert [r.rid for r in res] == [r.rid for r in reqs]
    assert rec["peak"] <= budget
    assert rec["max_running"] >= 2           # concurrency happened
    assert rec["order"] == sorted(rec["order"])  # first come, first served
    assert all(r.start >= r.arrival - 1e-6 for r in res)


def test_oversized_request_runs_alone():
    reqs = small_stream(count=4)
    rec = {"inflight": 0, "peak": 0, "running": 0, "max_running": 0, "order": []}
    serve.Server(budget_bytes=1.0, workers=4, solver=fake_solver(rec)).run(reqs)
    assert rec["max_running"] == 1


def test_one_at_a_time_is_sequential():
    reqs = small_stream(count=5)
    rec = {"inflight": 0, "peak": 0, "running": 0, "max_running": 0, "order": []}
    res = serve.one_at_a_time(reqs, solver=fake_solver(rec))
    assert rec["max_running"] == 1
    assert all(b.start >= a.finish for a, b in zip(res, res[1:]))
    s = serve.summary(res)
    assert s["requests"] == 5 and s["failed"] == 0 and s["p99_s"] >= s["p50_s"]


def fake_batch_solver(record, dt=0.02):
    lock = threading.Lock()

    def solve(reqs, device, keep):
        cost = sum(serve.BatchServer()._cost(r) for r in reqs)
        with lock:
            record["inflight"] += cost
            record["peak"] = max(record["peak"], record["inflight"])
            record["running"] += 1
            record["max_running"] = max(record["max_running"], record["running"])
            record["batches"].append([r.rid for r in reqs])
        time.sleep(dt)
        with lock:
            record["inflight"] -= cost
            record["running"] -= 1
        info = SimpleNamespace(iterations=1, refinements=0, true_residual=0.0, status=0)
        return [(info, 1, r.n ** 3, None) for r in reqs], 0.0

    return solve


def test_batch_server_forms_batches_within_budget():
    """Continuous batching: every request is served once; a batch holds one
    block edge and sizes within the ratio of its head, the oldest request
    waiting when it was formed; batches in flight stay within the budget;
    several run at once."""
    reqs = serve.poisson_stream(60, 2000.0, seed=7, cells=(1e4, 1e6), sizes=(8, 16),
                                levels=(2, 3))
    srv0 = serve.BatchServer()
    costs = sorted(srv0._cost(r) for r in reqs)
    budget = costs[-1] * 4
    rec = {"inflight": 0, "peak": 0, "running": 0, "max_running": 0, "batches": []}
    srv = serve.BatchServer(budget_bytes=budget, workers=3, size_ratio=4.0,
                            solver=fake_batch_solver(rec))
    res = srv.run(reqs)
    byid = {r.rid: r for r in reqs}
    assert sorted(r.rid for r in res) == [r.rid for r in reqs]
    seen = [rid for b in rec["batches"] for rid in b]
    assert sorted(seen) == sorted(byid)
    for b in rec["batches"]:
        head = byid[b[0]]
        assert all(byid[k].n == head.n for k in b)
        assert all(0.25 <= byid[k].target_cells / head.target_cells <= 4.0 for k in b)
    assert rec["peak"] <= budget
    assert rec["max_running"] >= 2
    assert max(len(b) for b in rec["batches"]) >= 2
    assert all(r.start >= r.arrival - 1e-6 for r in res)
    assert srv.batches == len(rec["batches"])
