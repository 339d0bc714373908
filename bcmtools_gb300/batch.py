"""Batched instances: many independent problems of one block edge and ghost
width solved as one block set.

The reference runs one BlockManager (one block list, one face list) per
problem (BlockManager.cpp:28-59, 471-530).  Here the blocks of many
instances are concatenated, with each instance's neighbour ids shifted by its
first block, into a single registration: the face table, the fused sweeps and
their CUDA-graph replays then cover all instances in every launch, and no
entry connects two instances, so each instance's values are those it would
get alone (bit for bit: every block sees the same neighbours and
coefficients).  `plan_block_sets` chooses the sets: L2-sized sets where a
cache-sized set still holds several waves of CTAs, one set streamed from HBM
for the rest (`chunk_for_cache`: in-order L2-sized chunks).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from .blockmanager import BC_DIRICHLET, DIRICHLET_SOR, BlockManager, laplace_coef


class Batch:
    """A block set made of `workloads` (objects with .tree, .n, .vc), all with
    the same block edge n and ghost width vc."""

    def __init__(self, workloads: Sequence, device: int = 0):
        if not workloads:
            raise ValueError("empty batch")
        n, vc = workloads[0].n, workloads[0].vc
        if any(w.n != n or w.vc != vc for w in workloads):
            raise ValueError("a batch holds one block edge and one ghost width")
        self.n, self.vc = n, vc
        self.workloads = list(workloads)
        lds, nids, sfs, outers, sizes = [], [], [], [], []
        self.first, self.count = [], []
        off = 0
        for w in workloads:
            ld, nid, sf, outer = w.tree.neighbors()
            nid = np.where(nid >= 0, nid + off, nid).astype(np.int32)
            lds.append(ld)
            nids.append(nid)
            sfs.append(sf)
            outers.append(outer)
            sizes.append(w.tree.cell_sizes(n))
            self.first.append(off)
            self.count.append(ld.shape[0])
            off += ld.shape[0]
        self.nb = off
        self.outer = np.concatenate(outers)
        self.cell_sizes = np.concatenate(sizes)
        self.bm = BlockManager(device)
        self.bm.register_blocks(np.concatenate(lds), np.concatenate(nids), np.concatenate(sfs), n)
        self.bm.outer = self.outer

    @classmethod
    def from_dividers(cls, specs: Sequence, n: int, vc: int = 1, device: int = 0) -> "Batch":
        """The batch of meshes [(rootgrid, divider), ...] made by the device
        set-up in one call (BlockManager.build_mesh_batch): octrees, balance,
        neighbour tables and face tables built on the GPU, no host tree."""
        self = cls.__new__(cls)
        self.n, self.vc = n, vc
        self.bm = BlockManager(device)
        self.first, meshes = self.bm.build_mesh_batch(specs, n)
        self.count = [m.num_leaves for m in meshes]
        self.workloads = [_DeviceInstance(m, n, vc) for m in meshes]
        self.nb = self.bm.nb
        self.outer = self.bm.outer
        self.cell_sizes = np.concatenate([m.cell_sizes(n) for m in meshes])
        return self

    @property
    def cells(self) -> int:
        return self.nb * self.n ** 3

    def set_dirichlet(self, value: float = 0.0, form=DIRICHLET_SOR):
        """Dirichlet on every outer face of every instance."""
        t = np.where(self.outer != 0, BC_DIRICHLET, 0).astype(np.int32)
        v = np.where(self.outer != 0, value, 0.0)
        self.bm.set_boundary(t, v, form)
        return t, v

    def laplace_op(self):
        return self.bm.op_const(laplace_coef(self.cell_sizes))

    def fill_rhs(self, field, seeds: Sequence[int], lo=-1.0, hi=1.0, stream=None):
        """Instance k's interior from fill_random(seeds[k]): the values the
        instance gets when registered alone with the same seed."""
        field.fill(0.0, stream=stream)
        for k, s in enumerate(seeds):
            field.fill_random(s, lo, hi, first_block=self.first[k], nblocks=self.count[k],
                              stream=stream)

    def set_segments(self):
        """Make every instance its own system for the BiCGSTAB solvers
        (bcmg_set_segments): one solve then advances all instances, each with
        its own scalars and convergence test."""
        self.bm.set_segments(list(self.first) + [self.nb])

    def instance(self, a: np.ndarray, k: int) -> np.ndarray:
        """Instance k's bricks in a host array of the whole batch."""
        return a[self.first[k]:self.first[k] + self.count[k]]


class _DeviceInstance:
    """One mesh of a device-built batch, with the attributes of a workload."""

    def __init__(self, tree, n: int, vc: int):
        self.tree, self.n, self.vc = tree, n, vc

    @property
    def nb(self) -> int:
        return self.tree.num_leaves


def group_by_shape(workloads: Sequence):
    """{(n, vc): [workloads]} preserving order."""
    groups = {}
    for w in workloads:
        groups.setdefault((w.n, w.vc), []).append(w)
    return groups


def brick_bytes(w, fields: int = 3, itemsize: int = 4) -> int:
    """Device bytes of `fields` fields of workload w (padded bricks)."""
    return w.nb * (w.n + 2 * w.vc) ** 3 * itemsize * fields


def chunk_for_cache(workloads: Sequence, cache_bytes: float, fields: int = 3,
                    itemsize: int = 4):
    """Instances of one block edge packed, in order, into chunks whose `fields`
    fields fit `cache_bytes` (GB300's 126 MB L2): a chunk's sweeps then run
    from the cache from the second one on.  An instance larger than the cache
    is a chunk of its own."""
    chunks, cur, used = [], [], 0
    for w in workloads:
        wb = brick_bytes(w, fields, itemsize)
        if cur and used + wb > cache_bytes:
            chunks.append(cur)
            cur, used = [], 0
        cur.append(w)
        used += wb
    if cur:
        chunks.append(cur)
    return chunks


def plan_block_sets(workloads: Sequence, cache_bytes: float, fields: int = 3,
                    itemsize: int = 4, min_set_blocks: int = 0):
    """Block sets for a batch of instances of one block edge, each set swept
    by one launch per iteration.  Instances whose `fields` fields fit
    `cache_bytes` are packed first-fit-decreasing into sets that fit it (their
    sweeps run from L2); all larger instances form one set together, whose
    sweeps stream from HBM anyway and gain from whole waves of CTAs (an
    instance of a few hundred 32^3 blocks alone fills less than one wave of
    152 SMs x 3 CTAs).  When the cache holds fewer than `min_set_blocks`
    blocks of this shape, cache-sized sets would be launch- and latency-bound
    (a few waves of CTAs a sweep): every instance then goes to the one set.
    Returns a list of lists of workloads, the large set last."""
    if not workloads:
        return []
    w0 = workloads[0]
    per_block = brick_bytes(w0, fields, itemsize) / max(1, w0.nb)
    if cache_bytes < min_set_blocks * per_block:
        return [list(workloads)]
    small, large = [], []
    for w in workloads:
        (small if brick_bytes(w, fields, itemsize) <= cache_bytes else large).append(w)
    sets, used = [], []
    for w in sorted(small, key=lambda w: -brick_bytes(w, fields, itemsize)):
        wb = brick_bytes(w, fields, itemsize)
        for k in range(len(sets)):
            if used[k] + wb <= cache_bytes:
                sets[k].append(w)
                used[k] += wb
                break
        else:
            sets.append([w])
            used.append(wb)
    if large:
        sets.append(large)
    return sets
