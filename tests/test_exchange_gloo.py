"""CPU, two gloo ranks: the exchange plan of a mesh split over processes.

Every rank holds the whole octree (as the reference's ranks do) and its
contiguous share of the leaves (Partition.h:46-108).  The faces a rank
receives from a peer must be listed by that peer as the faces it sends, in
the same order, with the same face, subface and kind, so that the buffers
line up (CommBuffer.cpp:146-203); each entry's size is the reference's
(getSendBufferByteSize and its F2C / C2F variants); and a rank's local
neighbour table keeps exactly its faces to its own blocks.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _mesh():
    from tests.helpers import small_octree
    return small_octree(level=3, radius=0.3)


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bcmtools_gb300 import exchange as X
    from bcmtools_gb300.mesh import Partition
    tree = _mesh()
    ld, nid, sf, _ = tree.neighbors()
    rank_of = Partition(world, tree.num_leaves).ranks()
    p = X.plan(ld, nid, sf, rank_of, rank)
    # the lists in global ids, gathered: (peer -> rows of (global block, f, s, kind))
    mine = {"send": {k: [(int(p.local[b]), f, s, kind) for b, f, s, kind in v]
                     for k, v in p.send.items()},
            "recv": {k: [(int(p.local[b]), f, s, kind) for b, f, s, kind in v]
                     for k, v in p.recv.items()},
            "local": p.local.tolist(), "lnid": p.nid.tolist()}
    allp = [None] * world
    dist.all_gather_object(allp, mine)
    out[rank] = allp
    dist.destroy_process_group()


def test_two_rank_exchange_plans_line_up():
    from bcmtools_gb300 import exchange as X
    from bcmtools_gb300.mesh import Partition
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    allp = res[0]
    tree = _mesh()
    ld, nid, sf, _ = tree.neighbors()
    rank_of = Partition(world, tree.num_leaves).ranks()
    faces = X.receiving_faces(ld, nid, sf)
    cross = [(b, f, s, k, src) for b, f, s, k, src in faces if rank_of[b] != rank_of[src]]
    assert cross, "the split must cut faces"
    n_send = n_recv = 0
    for r in range(world):
        for peer, rows in allp[r]["recv"].items():
            sent = allp[peer]["send"][r]
            assert len(sent) == len(rows)
            for (rb, f, s, k), (sb, f2, s2, k2) in zip(rows, sent):
                assert (f, s, k) == (f2, s2, k2)
                assert rank_of[rb] == r and rank_of[sb] == peer
                assert (rb, f, s, k, sb) in cross
            n_recv += len(rows)
        n_send += sum(len(v) for v in allp[r]["send"].values())
    assert n_send == n_recv == len(cross)
    # sizes: the reference's per-face buffers
    assert X.entry_values(8, 2, X.XCH_COPY, 4) == 2 * 8 * 8 * 4
    assert X.entry_values(8, 2, X.XCH_F2C, 8) == 2 * 4 * 4 * 8
    assert X.entry_values(8, 2, X.XCH_C2F, 4) == 2 * 8 * 8 * 4
    # local tables: own-block neighbours kept (renumbered), the others cut
    for r in range(world):
        local = np.array(allp[r]["local"])
        lnid = np.array(allp[r]["lnid"])
        g = nid[local]
        own = (g >= 0) & (rank_of[np.maximum(g, 0)] == r)
        assert np.array_equal(lnid >= 0, own)
        assert np.array_equal(local[lnid[own]], g[own])
