"""Ghost exchange between processes that each own part of one octree mesh.

The reference partitions the leaves over MPI ranks (Partition.h:46-108) and,
for every face whose neighbour lives on another rank, the sender fills a
communication buffer (Scalar3DUpdater::copyToCommBuffer*, the neighbour's
ghost values: copy, F2C average or C2F interpolation) which the receiver
copies into its ghosts (copyFromCommBuffer*), one buffer per peer holding its
faces in order (CommBuffer.cpp:146-203).  Here:

* `plan(ld, nid, sf, rank_of, rank)`: from the global neighbour table (every
  process holds the whole octree, as the reference's ranks do), this
  process's blocks (local ids in global order), their neighbour table with
  local ids (a neighbour on another process becomes -1, so the local face
  table leaves those faces to the exchange), and per peer the entries it
  sends and receives -- both sides list a peer's faces in the same order
  (receiving block's global id, face, subface), so the buffers line up.
* `Exchanger`: packs every peer's buffer on the device (bcmg_xch_pack),
  moves it (torch.distributed isend / irecv, or any transport), and unpacks
  the received ones into the ghosts (bcmg_xch_unpack).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict

import numpy as np

from . import capi

XCH_COPY, XCH_F2C, XCH_C2F = 0, 1, 2


@dataclass
class Plan:
    rank: int
    local: np.ndarray               # global ids of this process's blocks, local order
    ld: np.ndarray                  # local neighbour table (ids local, remote -> -1)
    nid: np.ndarray
    sf: np.ndarray
    # per peer: rows (local block, receiving face, subface, kind)
    send: Dict[int, np.ndarray] = field(default_factory=dict)
    recv: Dict[int, np.ndarray] = field(default_factory=dict)


def receiving_faces(ld, nid, sf):
    """Every (receiver, face, subface, kind, sender) the ghost update fills
    from a neighbour, in (receiver, face, subface) order."""
    ld = np.asarray(ld)
    nid = np.asarray(nid)
    sf = np.asarray(sf)
    out = []
    for b in range(ld.shape[0]):
        for f in range(6):
            l = int(ld[b, f])
            if l in (0, -1):
                s = int(nid[b, f, 0])
                if s >= 0:
                    out.append((b, f, int(sf[b, f]) if l == -1 else 0,
                                XCH_COPY if l == 0 else XCH_C2F, s))
            else:
                for q in range(4):
                    s = int(nid[b, f, q])
                    if s >= 0:
                        out.append((b, f, q, XCH_F2C, s))
    return out


def plan(ld, nid, sf, rank_of, rank: int) -> Plan:
    rank_of = np.asarray(rank_of)
    nb = len(rank_of)
    local = np.flatnonzero(rank_of == rank)
    g2l = np.full(nb, -1, np.int64)
    g2l[local] = np.arange(len(local))
    lld = np.ascontiguousarray(np.asarray(ld)[local], np.int32)
    g = np.asarray(nid)[local]
    mine = (g >= 0) & (rank_of[np.maximum(g, 0)] == rank)
    lnid = np.where(mine, g2l[np.maximum(g, 0)], -1).astype(np.int32)
    lsf = np.ascontiguousarray(np.asarray(sf)[local], np.int32)
    p = Plan(rank, local, lld, np.ascontiguousarray(lnid), lsf)
    send, recv = {}, {}
    for b, f, s, kind, src in receiving_faces(ld, nid, sf):
        rb, rs = int(rank_of[b]), int(rank_of[src])
        if rb == rs:
            continue
        if rs == rank:
            send.setdefault(rb, []).append((g2l[src], f, s, kind))
        if rb == rank:
            recv.setdefault(rs, []).append((g2l[b], f, s, kind))
    p.send = {k: np.array(v, np.int32).reshape(-1, 4) for k, v in send.items()}
    p.recv = {k: np.array(v, np.int32).reshape(-1, 4) for k, v in recv.items()}
    return p


def entry_values(n: int, vc: int, kind: int, itemsize: int) -> int:
    """Bytes of one entry's buffer (getSendBufferByteSize and its F2C / C2F
    variants, Scalar3DUpdater.h:84-111), cubic blocks of n cells."""
    return vc * (n // 2) ** 2 * itemsize if kind == XCH_F2C else vc * n * n * itemsize


def _entries(rows: np.ndarray):
    arr = (capi.XchEntryC * max(1, len(rows)))()
    for i, (b, f, s, k) in enumerate(rows):
        arr[i] = capi.XchEntryC(int(b), int(f), int(s), int(k))
    return arr, len(rows)


class Exchanger:
    """Device buffers of one field's exchange with every peer (torch uint8
    tensors on the field's device).  pack() fills the send buffers,
    unpack() empties the receive buffers into the ghosts; exchange() does
    both around torch.distributed isend / irecv (one message per peer)."""

    def __init__(self, bm, field, p: Plan):
        import torch
        self.bm, self.field, self.plan = bm, field, p
        lib = bm.lib
        self.send, self.recv = {}, {}
        for peer, rows in p.send.items():
            ents, n = _entries(rows)
            nbytes = C.c_size_t()
            bm._ck(lib.bcmg_xch_bytes(bm.ctx, field.id, ents, n, C.byref(nbytes)))
            buf = torch.empty(max(1, nbytes.value), dtype=torch.uint8, device=f"cuda:{bm.device}")
            self.send[peer] = (ents, n, buf, nbytes.value)
        for peer, rows in p.recv.items():
            ents, n = _entries(rows)
            nbytes = C.c_size_t()
            bm._ck(lib.bcmg_xch_bytes(bm.ctx, field.id, ents, n, C.byref(nbytes)))
            buf = torch.empty(max(1, nbytes.value), dtype=torch.uint8, device=f"cuda:{bm.device}")
            self.recv[peer] = (ents, n, buf, nbytes.value)

    def pack(self, stream=None):
        for ents, n, buf, _ in self.send.values():
            self.bm._ck(self.bm.lib.bcmg_xch_pack(self.bm.ctx, self.field.id, ents, n,
                                                  C.c_void_p(buf.data_ptr()), stream))

    def unpack(self, stream=None):
        for ents, n, buf, _ in self.recv.values():
            self.bm._ck(self.bm.lib.bcmg_xch_unpack(self.bm.ctx, self.field.id, ents, n,
                                                    C.c_void_p(buf.data_ptr()), stream))

    def exchange(self, group=None):
        """Pack, send every peer its buffer and receive theirs, unpack: the
        context's stream is synchronised before the messages, and the device
        after them (the messages run on the transport's own streams)."""
        import torch
        import torch.distributed as dist
        self.pack()
        self.bm.sync()
        reqs = [dist.isend(buf[:nb], peer, group=group)
                for peer, (_, _, buf, nb) in self.send.items() if nb]
        reqs += [dist.irecv(buf[:nb], peer, group=group)
                 for peer, (_, _, buf, nb) in self.recv.items() if nb]
        for r in reqs:
            r.wait()
        torch.cuda.synchronize(self.bm.device)
        self.unpack()
