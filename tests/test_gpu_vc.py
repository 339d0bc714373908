"""GPU: the ghost (VC) gather kernel through the C ABI.

Bar: bit-exact against the reference (golden fixtures) and against the
oracle for same-level copies, F2C averaging and C2F interpolation, in FP32
and FP64, vc = 1, 2, 3; edges and corners are never written.
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from oracle import pyoracle as po
from tests.helpers import (GOLDEN, assert_bitexact, assert_ghosts_match, edge_mask, face_mask,
                           outer_dirichlet,
                           small_octree, splitmix_uniform)

pytestmark = pytest.mark.gpu

VC_CASES = ["vc_f32_n4_vc1", "vc_f32_n4_vc2", "vc_f64_n4_vc1", "vc_f64_n4_vc2"]


def make_bm(tree, n, dtype, vc):
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    f = bm.setDataClass(dtype, vc)
    bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
    return bm, f


@pytest.mark.parametrize("name", VC_CASES)
def test_vc_matches_reference_golden(gpu_ok, name):
    g = np.load(GOLDEN / f"{name}.npz")
    dt = "f32" if "f32" in name else "f64"
    n, vc = int(g["n"]), int(g["vc"])
    rg = bg.RootGrid(2, 2, 2, periodic=(True, False, False), root_length=0.5)
    tree = bg.Octree.from_pedigrees(rg, g["pedigrees"])
    bm, f = make_bm(tree, n, dt, vc)
    a = splitmix_uniform(int(g["seed"]), f.shape[0] * np.prod(f.shape[1:])).reshape(f.shape)
    f.upload(a.astype(f.dtype))
    bm.beginUpdateVC(f)
    bm.endUpdateVC(f)
    assert_ghosts_match(f.download(), g["after"], what=name)


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("n,vc", [(8, 1), (8, 2), (8, 3), (16, 2)])
def test_vc_matches_oracle(gpu_ok, dt, n, vc):
    tree = small_octree(level=3, radius=0.3)
    bm, f = make_bm(tree, n, dt, vc)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    rng = np.random.default_rng(n * 10 + vc)
    a = rng.uniform(-1, 1, size=f.shape).astype(f.dtype)
    f.upload(a)
    bm.updateVC(f)
    got = f.download()
    ref = a.copy()
    m.vc_update(ref)
    assert_ghosts_match(got, ref, what=f"{dt} n={n} vc={vc}")


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_vc_partial_updates(gpu_ok, dt):
    """Per-axis and per-level-difference variants (updateVC_X_F2C etc.)."""
    n, vc = 8, 2
    tree = small_octree(level=3, radius=0.3)
    bm, f = make_bm(tree, n, dt, vc)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    rng = np.random.default_rng(3)
    a = rng.uniform(-1, 1, size=f.shape).astype(f.dtype)
    for axis_mask, ld_mask in [(1, 7), (2, 4), (4, 1), (3, 2), (5, 5)]:
        f.upload(a)
        bm.updateVC(f, axis_mask, ld_mask)
        ref = a.copy()
        m.vc_update(ref, axis_mask, ld_mask)
        assert_ghosts_match(f.download(), ref, what=f"mask {axis_mask},{ld_mask}")
    f.upload(a)
    for xyz in range(3):
        bm.updateVC_F2C(f, xyz)
    for xyz in range(3):
        bm.updateVC_Flat(f, xyz)
    for xyz in range(3):
        bm.updateVC_C2F(f, xyz)
    ref = a.copy()
    m.vc_update(ref)
    assert_ghosts_match(f.download(), ref, what="separate level diff")


def test_vc_leaves_edges_and_corners(gpu_ok):
    n, vc = 8, 2
    tree = small_octree(level=3, radius=0.3)
    bm, f = make_bm(tree, n, "f64", vc)
    a = np.full(f.shape, np.nan)
    a[:, face_mask(n, vc)] = np.random.default_rng(1).uniform(size=(f.shape[0], face_mask(n, vc).sum()))
    f.upload(a)
    bm.updateVC(f)
    got = f.download()
    assert np.isnan(got[:, edge_mask(n, vc)]).all()
    assert not np.isnan(got[:, face_mask(n, vc)]).any()


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("form", [bg.DIRICHLET_SOR, bg.DIRICHLET_BCX])
def test_dirichlet_and_impose(gpu_ok, dt, form):
    n, vc = 8, 2
    tree = small_octree(periodic=(True, False, False), level=3, radius=0.3)
    bm, f = make_bm(tree, n, dt, vc)
    bct, bcv = outer_dirichlet(tree, 0.37, periodic=(True, False, False))
    bm.set_boundary(bct, bcv, form)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    a = np.random.default_rng(9).uniform(-1, 1, size=f.shape).astype(f.dtype)
    f.upload(a)
    bm.setBoundaryCondition(f)
    ref = a.copy()
    m.dirichlet(ref, bct, bcv, form)
    assert_bitexact(f.download(), ref, what="bc only")
    f.upload(a)
    bm.imposeBoundaryCondition(f)
    ref = a.copy()
    m.vc_update(ref)
    m.dirichlet(ref, bct, bcv, form)
    assert_ghosts_match(f.download(), ref, what="impose")


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("vc", [1, 2])
def test_neumann_and_impose(gpu_ok, dt, vc):
    """Neumann ghosts (SolverTest/bcx.f90:198-376) on the outer y and z faces
    beside Dirichlet ones on x: bit-exact against the oracle, alone and after
    a VC update."""
    n = 8
    tree = small_octree(periodic=(False, False, False), level=2, radius=0.3)
    bm, f = make_bm(tree, n, dt, vc)
    bct, bcv = outer_dirichlet(tree, 0.37, periodic=(False, False, False))
    bct[:, 2:6] = np.where(bct[:, 2:6] != 0, bg.BC_NEUMANN, 0)
    bcv[:, 2:6] = np.random.default_rng(4).uniform(-0.05, 0.05, size=(bct.shape[0], 4))
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    a = np.random.default_rng(10).uniform(-1, 1, size=f.shape).astype(f.dtype)
    f.upload(a)
    bm.setBoundaryCondition(f)
    ref = a.copy()
    m.dirichlet(ref, bct, bcv, 0)
    assert_bitexact(f.download(), ref, what="neumann bc only")
    f.upload(a)
    bm.imposeBoundaryCondition(f)
    ref = a.copy()
    m.vc_update(ref)
    m.dirichlet(ref, bct, bcv, 0)
    assert_ghosts_match(f.download(), ref, what="neumann impose")


def test_vc_two_level_sphere_full_size(gpu_ok):
    """The benchmark mesh (4432 blocks of 16^3, vc=2), FP32, against the oracle."""
    from bcmtools_gb300 import workloads as W
    w = W.two_level_sphere()
    bm, f = make_bm(w.tree, w.n, "f32", w.vc)
    ld, nid, sf, _ = w.neighbors()
    m = po.OracleMesh(ld, nid, sf, w.n, w.vc)
    a = np.random.default_rng(11).uniform(-1, 1, size=f.shape).astype(np.float32)
    f.upload(a)
    bm.updateVC(f)
    ref = a.copy()
    m.vc_update(ref)
    assert_ghosts_match(f.download(), ref, what="two_level_sphere")
