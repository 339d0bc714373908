"""Runs oracle/_ref/refbench, the reference's own OpenMP CPU path of the
red-black SOR benchmark (sor2's Solver sweep and Dirichlet code with the
reference BlockManager's ghost update; see refbench.cpp).  Test and benchmark
infrastructure only: the CPU leg of bench.py and the CPU tests use it.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BINARY = HERE / "_ref" / "refbench"


def available() -> bool:
    return BINARY.is_file() and os.access(BINARY, os.X_OK)


def run(tree, n: int, vc: int, s: np.ndarray, omega: float, threads: int, warmup: int,
        iters: int, timeout: float = 600.0):
    """Times `iters` iterations (after `warmup`) of the reference path on the
    mesh of `tree` with source bricks `s` (float64, packed, block order of
    `tree`) from f = 0.  Returns (seconds, f) with f the final field in the
    block order of `tree` (the reference numbers the same pedigree list's
    blocks in its own order; they are matched back by pedigree)."""
    rg = tree.rootgrid
    peds = np.ascontiguousarray(tree.pedigrees, dtype=np.uint64)
    nb = len(peds)
    s = np.ascontiguousarray(s, dtype=np.float64)
    n0 = n + 2 * vc
    assert s.shape == (nb, n0, n0, n0)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fp:
            fp.write(np.array([rg.nx, rg.ny, rg.nz, n, vc, nb], np.int32).tobytes())
            fp.write(np.array([rg.root_length, omega], np.float64).tobytes())
            fp.write(peds.tobytes())
            fp.write(s.tobytes())
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        subprocess.run([str(BINARY), str(fin), str(threads), str(warmup), str(iters), str(fout)],
                       check=True, env=env, timeout=timeout)
        raw = fout.read_bytes()
    sec = float(np.frombuffer(raw, np.float64, 1, 0)[0])
    nl = int(np.frombuffer(raw, np.int32, 1, 8)[0])
    rec = np.dtype([("ped", "<u8"), ("f", "<f8", (n0, n0, n0))])
    out = np.frombuffer(raw, rec, nl, 12)
    order = {int(p): i for i, p in enumerate(out["ped"])}
    f = np.stack([out["f"][order[int(p)]] for p in peds])
    return sec, f
