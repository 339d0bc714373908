"""CPU, two gloo ranks: the bench's multi-GPU aggregation (one independent
replica per rank, no collective on the data path; the timing is the slowest
rank's and the value counts every rank's cells)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    assert bench.dist_env() == (world, rank, rank)
    ms = [120.0, 150.0][rank]  # rank 1 is the slow one
    dist.barrier()
    ms_max = bench.max_over_ranks(ms, dist, "cpu")
    value = bench.whole_job_rate(1000, 10, 2, world, ms_max)
    out[rank] = (ms_max, value)
    dist.destroy_process_group()


def test_two_rank_replicas_aggregate():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms_max, value = res[0]
    assert ms_max == 150.0
    assert abs(value - 1000 * 10 * 2 * 2 / 0.150 / 1e9) < 1e-15
