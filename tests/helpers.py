"""Shared helpers for the parity tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def splitmix_uniform(seed: int, n: int) -> np.ndarray:
    """Seeded fill used by the golden-fixture driver (oracle/refvc.cpp)."""
    golden = np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        s = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * golden
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def face_mask(n: int, vc: int) -> np.ndarray:
    """Cells of a brick that lie in at most one ghost slab (interior + faces);
    edges and corners are never written by the reference."""
    k = np.arange(n + 2 * vc)
    g = ((k < vc) | (k >= n + vc)).astype(int)
    return (g[:, None, None] + g[None, :, None] + g[None, None, :]) <= 1


def edge_mask(n: int, vc: int) -> np.ndarray:
    return ~face_mask(n, vc)


def bits(a: np.ndarray) -> np.ndarray:
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def assert_bitexact(got: np.ndarray, ref: np.ndarray, mask=None, what=""):
    g, r = (got, ref) if mask is None else (got[:, mask], ref[:, mask])
    diff = bits(np.ascontiguousarray(g)) != bits(np.ascontiguousarray(r))
    n = int(diff.sum())
    if n:
        idx = np.argwhere(diff)[:5]
        raise AssertionError(f"{what}: {n} cells differ (first {idx.tolist()}); "
                             f"max abs {np.abs(g.astype(np.float64) - r).max():.3e}")


def assert_ghosts_match(got: np.ndarray, ref: np.ndarray, what=""):
    """Ghost-update parity: FP64 bit-exact; FP32 within one ulp (the C2F
    interpolation of FP32 fields is evaluated in float-float, bit-exact except
    next to rounding boundaries), everything else bit-exact."""
    if got.dtype == np.float64:
        assert_bitexact(got, ref, what=what)
        return
    u = ulp_diff(got, ref)
    assert int(u.max()) <= 1, f"{what}: max ulp difference {int(u.max())}"
    assert (u != 0).mean() < 1e-4, f"{what}: {(u != 0).sum()} cells differ by one ulp"


def assert_close_normwise(got, ref, tol, mask=None, what=""):
    g = got if mask is None else got[:, mask]
    r = ref if mask is None else ref[:, mask]
    err = np.abs(g.astype(np.float64) - r.astype(np.float64)).max()
    scale = np.abs(r.astype(np.float64)).max()
    assert err <= tol * scale, f"{what}: max abs diff {err:.3e} > {tol:.1e} x {scale:.3e}"


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ia = bits(np.ascontiguousarray(a)).astype(np.int64)
    ib = bits(np.ascontiguousarray(b)).astype(np.int64)
    return np.abs(ia - ib)


def small_octree(periodic=(True, False, False), level=2, radius=0.32):
    import bcmtools_gb300 as bg
    rg = bg.RootGrid(2, 2, 2, periodic=periodic, root_length=0.5)
    return bg.Octree.build(rg, bg.Divider.sphere_surface((0.5, 0.5, 0.5), radius, level), "Z")


def outer_dirichlet(tree, value=0.0, periodic=(False, False, False)):
    _, _, _, outer = tree.neighbors()
    t = (outer != 0).astype(np.int32)
    for ax in range(3):
        if periodic[ax]:
            t[:, 2 * ax:2 * ax + 2] = 0
    v = np.where(t != 0, value, 0.0)
    return t, v
