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
