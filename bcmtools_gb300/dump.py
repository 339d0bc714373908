"""Per-block dump files for checkpoint / restart of a field.

The reference's format (SolverTest LocalScalar3D<real>::Dump / Load,
examples/SolverTest/LocalScalar3D.cpp:85-222): one file per block,
``<dir>/dump-<label>-<rank:05>-<block:05>-<step:010>.bin``, holding five
native int32 values (nx, ny, nz, vc, 1) and then the block's padded brick
(nx+2vc)(ny+2vc)(nz+2vc) values of the field's element type, x fastest --
the host brick layout of `Scalar3D.download`.  A restart from files whose
blocks have half the cells per axis fills each cell with the value of the
coarse cell that contains it (bsf3d.f90:18-46, sf3d_copy_x2), ghosts
excepted; the caller then imposes the boundary conditions, as the
reference's Load does.
"""
from __future__ import annotations

import os
from typing import Tuple

import numpy as np


def dump_path(directory: str, label: str, rank: int, block: int, step: int) -> str:
    return os.path.join(directory, f"dump-{label}-{rank:05d}-{block:05d}-{step:010d}.bin")


def write_blocks(bricks: np.ndarray, vc: int, directory: str, label: str, step: int,
                 rank: int = 0) -> None:
    """One file per block of `bricks` (shape (nb, nz+2vc, ny+2vc, nx+2vc))."""
    nb, cz, cy, cx = bricks.shape
    n = (cx - 2 * vc, cy - 2 * vc, cz - 2 * vc)
    if min(n) < 1:
        raise ValueError("bricks narrower than their ghost layers")
    os.makedirs(directory, mode=0o755, exist_ok=True)
    head = np.array([n[0], n[1], n[2], vc, 1], dtype=np.int32)
    for b in range(nb):
        with open(dump_path(directory, label, rank, b, step), "wb") as f:
            f.write(head.tobytes())
            f.write(np.ascontiguousarray(bricks[b]).tobytes())


def _read_one(path: str, dtype) -> Tuple[Tuple[int, int, int], int, np.ndarray]:
    with open(path, "rb") as f:
        head = np.frombuffer(f.read(20), dtype=np.int32)
        if head.size != 5 or head[4] != 1:
            raise ValueError(f"{path}: not a one-component block dump")
        nx, ny, nz, vc = (int(v) for v in head[:4])
        cnt = (nx + 2 * vc) * (ny + 2 * vc) * (nz + 2 * vc)
        data = np.frombuffer(f.read(cnt * np.dtype(dtype).itemsize), dtype=dtype)
    if data.size != cnt:
        raise ValueError(f"{path}: truncated")
    return (nx, ny, nz), vc, data.reshape(nz + 2 * vc, ny + 2 * vc, nx + 2 * vc)


def read_blocks(shape, vc: int, directory: str, label: str, step: int, rank: int = 0,
                dtype=np.float32, out: np.ndarray | None = None) -> np.ndarray:
    """Bricks of shape `shape` (nb, nz+2vc, ny+2vc, nx+2vc) from the files:
    equal blocks are read as they are; blocks with half the cells per axis
    (same vc) fill the interior by injection and leave `out`'s ghosts."""
    nb, cz, cy, cx = shape
    n = (cx - 2 * vc, cy - 2 * vc, cz - 2 * vc)
    a = np.zeros(shape, dtype) if out is None else out
    for b in range(nb):
        fn, fvc, data = _read_one(dump_path(directory, label, rank, b, step), dtype)
        if fvc != vc:
            raise ValueError(f"block {b}: ghost width {fvc} in the file, {vc} in the field")
        if fn == n:
            a[b] = data
        elif tuple(2 * v for v in fn) == n:
            v = vc
            coarse = data[v:v + fn[2], v:v + fn[1], v:v + fn[0]]
            a[b, v:v + n[2], v:v + n[1], v:v + n[0]] = (
                coarse.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2))
        else:
            raise ValueError(f"block {b}: {fn} cells in the file, {n} in the field")
    return a
