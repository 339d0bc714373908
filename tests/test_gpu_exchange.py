"""GPU: ghost exchange through the reference's communication buffers.

A mesh split over two "processes" -- two contexts in this process, each
registering its share of the blocks with its local neighbour table -- must
end a ghost update with every ghost equal to the single-context update of
the whole mesh (and so to the oracle), bit for bit: local faces by each
context's own update, faces across the split by pack on the sender
(copy, F2C average, C2F interpolation computed there), a buffer copy, and
unpack on the receiver (Scalar3DUpdater.h:377-515, 711-901).  Each buffer
has the reference's size.
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import exchange as X
from bcmtools_gb300.mesh import Partition
from oracle import pyoracle as po
from tests.helpers import assert_ghosts_match, small_octree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("n,vc", [(8, 1), (8, 2), (16, 2)])
@pytest.mark.parametrize("world", [2, 3])
def test_split_mesh_exchange_equals_whole_update(gpu_ok, dt, n, vc, world):
    import torch
    tree = small_octree(level=3, radius=0.3)
    ld, nid, sf, _ = tree.neighbors()
    nb = tree.num_leaves
    rank_of = Partition(world, nb).ranks()
    npdt = np.float32 if dt == "f32" else np.float64
    shape = (nb, n + 2 * vc, n + 2 * vc, n + 2 * vc)
    a = np.random.default_rng(n * 10 + vc).uniform(-1, 1, size=shape).astype(npdt)
    ref = a.copy()
    po.OracleMesh(ld, nid, sf, n, vc).vc_update(ref)
    plans = [X.plan(ld, nid, sf, rank_of, r) for r in range(world)]
    bms, fields, xs = [], [], []
    for r, p in enumerate(plans):
        bm = bg.BlockManager(0)
        bm.register_blocks(p.ld, p.nid, p.sf, n)
        f = bm.setDataClass(dt, vc)
        bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
        f.upload(np.ascontiguousarray(a[p.local]))
        bm.updateVC(f)  # the faces inside this share
        bms.append(bm)
        fields.append(f)
        xs.append(X.Exchanger(bm, f, p))
    cut = 0
    for r, x in enumerate(xs):
        x.pack()
        bms[r].sync()
        for peer, (_, cnt, buf, nbytes) in x.send.items():
            rows = plans[r].send[peer]
            assert nbytes == sum(X.entry_values(n, vc, int(k), np.dtype(npdt).itemsize)
                                 for k in rows[:, 3])
            dst = xs[peer].recv[r]
            assert dst[3] == nbytes and dst[1] == cnt
            dst[2][:nbytes].copy_(buf[:nbytes])
            cut += cnt
    torch.cuda.synchronize()
    assert cut > 0
    for r, x in enumerate(xs):
        x.unpack()
        bms[r].sync()
        got = fields[r].download()
        assert_ghosts_match(got, ref[plans[r].local], what=f"rank {r} of {world}, {dt} n={n} vc={vc}")
