"""Host-side octree of blocks (mirror of the reference's Utils: RootGrid,
Divider family, BCMOctree).  Pure host code in libbcmg.so; needs no GPU.

Pedigrees use the reference's 64-bit packing (Utils/include/Pedigree.h:52-60):
x:16 | y:16 | z:16 | rootID:12 | level:4.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi

ORDERINGS = {"Z": 0, "HILBERT": 1, "RANDOM": 2}


def pedigree(level: int, x: int, y: int, z: int, root: int = 0) -> int:
    return (x << 48) | (y << 32) | (z << 16) | (root << 4) | level


def unpack_pedigrees(p: np.ndarray):
    p = np.asarray(p, dtype=np.uint64)
    return ((p & 0xF).astype(np.int64), ((p >> 48) & 0xFFFF).astype(np.int64),
            ((p >> 32) & 0xFFFF).astype(np.int64), ((p >> 16) & 0xFFFF).astype(np.int64),
            ((p >> 4) & 0xFFF).astype(np.int64))


class Partition:
    """Contiguous split of n_items over n_procs (Utils/include/Partition.h:
    33-108): the first n_items % n_procs ranks take one item more."""

    def __init__(self, n_procs: int, n_items: int):
        if n_procs < 1 or n_items < 0:
            raise ValueError("bad partition")
        m, r = divmod(n_items, n_procs)
        self.n_procs, self.n_items = n_procs, n_items
        self.end = np.cumsum([m + 1 if i < r else m for i in range(n_procs)]).astype(np.int64)

    def getStart(self, rank: int) -> int:
        return 0 if rank == 0 else int(self.end[rank - 1])

    def getEnd(self, rank: int) -> int:
        return int(self.end[rank])

    def getNum(self, rank: int) -> int:
        return self.getEnd(rank) - self.getStart(rank)

    def getRank(self, i: int) -> int:
        """Owner of item i; -1 (MPI::PROC_NULL's role) outside [0, n_items)."""
        if i < 0 or i >= self.n_items:
            return -1
        return int(np.searchsorted(self.end, i, side="right"))

    def ranks(self) -> np.ndarray:
        """Owner of every item."""
        return np.repeat(np.arange(self.n_procs), np.diff(np.concatenate([[0], self.end])))


def layout_info(levels, ld, nid, ranks=None) -> dict:
    """The counts of BlockManager::printBlockLayoutInfo (BlockManager.cpp:
    118-288): blocks per level, and faces with a neighbour by level
    difference -- one per face at 0 and -1, one per subface at +1 -- split
    into intra-rank and inter-rank by `ranks` (the rank of every block; all
    blocks on one rank when None)."""
    levels = np.asarray(levels)
    ld = np.asarray(ld)
    nid = np.asarray(nid).reshape(ld.shape[0], 6, 4)
    rank = np.zeros(ld.shape[0], np.int64) if ranks is None else np.asarray(ranks)
    intra = np.zeros(3, np.int64)  # level difference -1, 0, +1
    inter = np.zeros(3, np.int64)
    for d in (-1, 0, 1):
        nsub = 4 if d == 1 else 1
        sel = (ld == d)[:, :, None] & (nid[:, :, :nsub] >= 0)
        b, _, s = np.nonzero(sel)
        other = nid[:, :, :nsub][sel]
        same = rank[other] == rank[b]
        intra[d + 1] = int(same.sum())
        inter[d + 1] = int((~same).sum())
    lv, cnt = np.unique(levels, return_counts=True)
    return {"level_min": int(lv.min()), "level_max": int(lv.max()),
            "blocks": {int(l): int(c) for l, c in zip(lv, cnt)}, "total": int(levels.size),
            "faces_intra": intra.tolist(), "faces_inter": inter.tolist()}


def format_layout_info(info: dict) -> str:
    """printBlockLayoutInfo's text for one rank (BlockManager.cpp:118-288)."""
    lines = ["Block Layout Information", f"  Min level: {info['level_min']}",
             f"  Max level: {info['level_max']}", "  Number of blocks"]
    for l in range(info["level_min"], info["level_max"] + 1):
        lines.append(f"    L={l}: {info['blocks'].get(l, 0)}")
    lines.append(f"    total: {info['total']}")
    lines.append("  Number of faces")
    for name, v in (("intra-node ", info["faces_intra"]), ("inter-node ", info["faces_inter"])):
        lines += [f"    {name}", f"        dLevel=-1: {v[0]}", f"        dLevel= 0: {v[1]}",
                  f"        dLevel=+1: {v[2]}", f"            total: {sum(v)}"]
    return "\n".join(lines)


@dataclass
class RootGrid:
    """RootGrid(nx, ny, nz) with setPeriodicX/Y/Z (Utils/include/RootGrid.h)."""
    nx: int = 1
    ny: int = 1
    nz: int = 1
    periodic: tuple = (False, False, False)
    origin: tuple = (0.0, 0.0, 0.0)
    root_length: float = 1.0

    def to_c(self) -> capi.RootGridC:
        m = sum(1 << a for a in range(3) if self.periodic[a])
        return capi.RootGridC(self.nx, self.ny, self.nz, m, (C.c_double * 3)(*self.origin),
                              float(self.root_length))

    def size(self) -> int:
        return self.nx * self.ny * self.nz


@dataclass
class Divider:
    kind: int
    min_level: int = 0
    max_level: int = 0
    direction_mask: int = 0
    center: tuple = (0.0, 0.0, 0.0)
    radius: float = 0.0
    points: np.ndarray | None = None
    balance: bool = True
    margin_ratio: float = 0.0
    _keep: list = field(default_factory=list, repr=False)

    @staticmethod
    def flat(max_level: int) -> "Divider":
        """FlatDivider (Utils/include/SimpleDivider.h:30-64)."""
        return Divider(0, 0, max_level)

    @staticmethod
    def simple(min_level: int, max_level: int, direction_mask: int = 0) -> "Divider":
        """SimpleDivider (Utils/include/SimpleDivider.h:67-150); 0 = ALL faces."""
        return Divider(1, min_level, max_level, direction_mask)

    @staticmethod
    def sphere_surface(center, radius: float, max_level: int, min_level: int = 0) -> "Divider":
        """Refine blocks whose box meets the sphere surface; all leaves active."""
        return Divider(2, min_level, max_level, 0, tuple(center), float(radius))

    @staticmethod
    def sphere(center, radius: float, min_level: int, max_level: int,
               margin_ratio: float = 0.0) -> "Divider":
        """SphereDivider (Utils/include/SphereDivider.h:28-150): blocks inside
        the sphere become inactive leaves (no block), blocks meeting its
        surface divide to max_level, with the reference's ripple margin and
        float arithmetic; `margin_ratio` widens every search box by that
        fraction of a max_level block (extraMarginRatio).  Unbalanced, as in
        the reference.  `center` and `radius` are in root-index units (unit
        root blocks, root 0 at the origin), whatever the root grid's origin
        and root length: the reference builds this divider over origin 0 and
        root length 1 (SphereDivider.h:72)."""
        return Divider(4, min_level, max_level, 0, tuple(center), float(radius), balance=False,
                       margin_ratio=float(margin_ratio))

    @staticmethod
    def cylinder(center_xy, radius: float, min_level: int, max_level: int,
                 margin_ratio: float = 0.0) -> "Divider":
        """CylinderDivider (Utils/include/CylinderDivider.h:28-153): the
        sphere's tests on x and y around an axis along z; blocks outside the
        cylinder become inactive leaves.  Unbalanced, as in the reference.
        Center and radius in root-index units, as for `sphere`
        (CylinderDivider.h:69)."""
        cx, cy = center_xy
        return Divider(5, min_level, max_level, 0, (float(cx), float(cy), 0.0), float(radius),
                       balance=False, margin_ratio=float(margin_ratio))

    @staticmethod
    def balls(points, radius: float, max_level: int, min_level: int = 0) -> "Divider":
        """Refine blocks whose box meets any ball (point, radius)."""
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        return Divider(3, min_level, max_level, 0, (0.0, 0.0, 0.0), float(radius), pts)

    def to_c(self) -> capi.DividerC:
        d = capi.DividerC()
        d.kind, d.min_level, d.max_level = self.kind, self.min_level, self.max_level
        d.direction_mask = self.direction_mask
        d.center = (C.c_double * 3)(*self.center)
        d.radius = self.radius
        if self.points is not None:
            d.points = capi.ptr(self.points, C.c_double)
            d.npoints = len(self.points)
            self._keep = [self.points]
        d.balance = 1 if self.balance else 0
        d.margin_ratio = self.margin_ratio
        return d


class Octree:
    """BCMOctree (Utils/include/BCMOctree.h): leaves in block-id order and
    their NeighborInfo tables."""

    def __init__(self, handle, rootgrid: RootGrid):
        self._lib = capi.load()
        self._h = handle
        self.rootgrid = rootgrid
        n = C.c_int()
        self._check(self._lib.bcmg_octree_num_leaves(self._h, C.byref(n)))
        self.num_leaves = n.value
        nb = self.num_leaves
        self.pedigrees = np.zeros(nb, np.uint64)
        self.levels = np.zeros(nb, np.int32)
        self.origins = np.zeros((nb, 3), np.float64)
        self.block_sizes = np.zeros(nb, np.float64)
        self._check(self._lib.bcmg_octree_leaves(
            self._h, capi.ptr(self.pedigrees, C.c_uint64), capi.ptr(self.levels, C.c_int),
            capi.ptr(self.origins, C.c_double), capi.ptr(self.block_sizes, C.c_double)))

    @staticmethod
    def _check(rc):
        if rc != 0:
            raise capi.BcmgError(rc, "octree call failed")

    @classmethod
    def build(cls, rg: RootGrid, div: Divider, ordering: str = "Z", seed: int = 0) -> "Octree":
        lib = capi.load()
        h = C.c_void_p()
        rgc, dc = rg.to_c(), div.to_c()
        rc = lib.bcmg_octree_build(C.byref(h), C.byref(rgc), C.byref(dc),
                                   ORDERINGS[ordering.upper()], seed)
        if rc != 0:
            raise capi.BcmgError(rc, "bcmg_octree_build")
        return cls(h, rg)

    @classmethod
    def from_pedigrees(cls, rg: RootGrid, peds) -> "Octree":
        lib = capi.load()
        p = np.ascontiguousarray(np.asarray(peds, dtype=np.uint64))
        h = C.c_void_p()
        rgc = rg.to_c()
        rc = lib.bcmg_octree_from_pedigrees(C.byref(h), C.byref(rgc),
                                            capi.ptr(p, C.c_uint64), len(p))
        if rc != 0:
            raise capi.BcmgError(rc, "bcmg_octree_from_pedigrees")
        return cls(h, rg)

    def neighbors(self):
        """(ld[nb,6], id[nb,6,4], sf[nb,6], outer[nb,6]) as int32 arrays."""
        nb = self.num_leaves
        ld = np.zeros((nb, 6), np.int32)
        nid = np.zeros((nb, 6, 4), np.int32)
        sf = np.zeros((nb, 6), np.int32)
        outer = np.zeros((nb, 6), np.int32)
        rc = self._lib.bcmg_octree_neighbors(self._h, capi.ptr(ld, C.c_int),
                                             capi.ptr(nid, C.c_int), capi.ptr(sf, C.c_int),
                                             capi.ptr(outer, C.c_int))
        if rc != 0:
            raise capi.BcmgError(rc, "2:1 constraint is broken (BCMOctree.cpp:462-468)")
        return ld, nid, sf, outer

    def cell_sizes(self, n: int) -> np.ndarray:
        """BlockBase cellSize = blockSize / size (BlockBase.h:72-74)."""
        return np.repeat((self.block_sizes / n)[:, None], 3, axis=1)

    def __del__(self):
        try:
            if self._h:
                self._lib.bcmg_octree_destroy(self._h)
                self._h = None
        except Exception:
            pass


class DeviceMesh:
    """A mesh made by the device set-up (BlockManager.build_mesh,
    build_mesh_batch, register_pedigrees): its leaves and neighbour table as
    the Octree attributes the rest of the package reads (pedigrees, levels,
    origins, block sizes, num_leaves, neighbors(), cell_sizes())."""

    def __init__(self, rootgrid: RootGrid, pedigrees, ld, nid, sf, outer):
        self.rootgrid = rootgrid
        self.pedigrees = np.ascontiguousarray(pedigrees, np.uint64)
        self.num_leaves = len(self.pedigrees)
        lv, x, y, z, r = unpack_pedigrees(self.pedigrees)
        self.levels = lv.astype(np.int32)
        self.block_sizes = rootgrid.root_length / np.exp2(lv)
        rg = rootgrid
        ri = np.stack([r % rg.nx, (r // rg.nx) % rg.ny, r // (rg.nx * rg.ny)], axis=1)
        c = np.stack([x, y, z], axis=1)
        self.origins = (np.asarray(rg.origin, np.float64) + ri * rg.root_length
                        + c * self.block_sizes[:, None])
        self._nbr = (ld, nid, sf, outer)

    def neighbors(self):
        """(ld[nb,6], id[nb,6,4], sf[nb,6], outer[nb,6]) as int32 arrays."""
        return tuple(a.copy() for a in self._nbr)

    def cell_sizes(self, n: int) -> np.ndarray:
        """BlockBase cellSize = blockSize / size (BlockBase.h:72-74)."""
        return np.repeat((self.block_sizes / n)[:, None], 3, axis=1)
