"""GPU: red-black SOR (sor1 / sor2 schemes) through the C ABI.

Bar: FP64 bit-exact against the reference's sor1 run on its shipped
test.conf (errorMax = 0.00353051, examples/sor1/log.4:54) and against the
oracle for the sor2 scheme with a source, fused and unfused; FP32 (swept in
FP32 arithmetic) within 1e-6 relative (normwise, max |diff| / max |ref|) per
sweep of the oracle's double-evaluated expression; the fused ping-pong path
identical bit for bit to the separate sweep + gather path.
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from oracle import pyoracle as po
from tests.helpers import (GOLDEN, assert_bitexact, assert_close_normwise, face_mask,
                           outer_dirichlet, small_octree)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["pull", "push", "unfused"])
def test_sor1_known_answer(gpu_ok, mode):
    """sor1 on its shipped test.conf: the pull and push ghost forms of the
    fused sweep and the separate launches all give the reference's field."""
    g = np.load(GOLDEN / "sor1.npz")
    n, vc = int(g["n"]), int(g["vc"])
    rg = bg.RootGrid(1, 1, 1, periodic=(False, True, True))
    tree = bg.Octree.from_pedigrees(rg, g["pedigrees"])
    bm = bg.BlockManager(0)
    bm.set_fusion(mode != "unfused")
    bm.set_ghost_form(push=mode == "push")
    bm.register_octree(tree, n)
    bct = np.where(g["bc_type"] == 1, 1, 0).astype(np.int32)
    bcv = np.where(g["bc_id"] == 1, float(g["b1"]), float(g["b0"]))
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    f = bm.setDataClass("f64", vc)
    bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
    f.fill(0.0)
    bm.imposeBoundaryCondition(f)  # Solver::initialize
    coef = bg.sor1_coef(g["cell_sizes"], float(g["omega"]))
    bm.sor_run(f, coef, float(g["omega"]), form=1, n_inner=int(g["n_inner"]),
               n_outer=int(g["n_outer"]))
    got = f.download()
    assert_bitexact(got, g["field"], face_mask(n, vc), "sor1 vs reference")
    xs = g["origins"][:, 0, None] + (np.arange(n) + 0.5)[None, :] * g["cell_sizes"][:, 0, None]
    err = np.abs(got[:, vc:-vc, vc:-vc, vc:-vc] - xs[:, None, None, :]).max()
    assert f"{err:.6g}" == "0.00353051"


def run_sor2(dt, n, vc, n_inner, iters, fused, level=2, variant=0):
    tree = small_octree(periodic=(False, False, False), level=level, radius=0.3)
    bm = bg.BlockManager(0)
    bm.set_fusion(fused)
    bm.set_sor_variant(variant)
    bm.register_octree(tree, n)
    bct, bcv = outer_dirichlet(tree, 0.0)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    f = bm.setDataClass(dt, vc)
    s = bm.setDataClass(dt, vc)
    bm.prepareForVCUpdate(f)
    rng = np.random.default_rng(n + vc)
    a = np.zeros(f.shape, f.dtype)
    src = rng.uniform(-1, 1, size=f.shape).astype(f.dtype)
    f.upload(a)
    s.upload(src)
    bm.imposeBoundaryCondition(f)
    coef = bg.sor2_coef(tree.cell_sizes(n))
    bm.sor_run(f, coef, 1.8, form=2, n_inner=n_inner, n_outer=iters, s=s)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    ref = a.copy()
    m.vc_update(ref)
    m.dirichlet(ref, bct, bcv, 0)
    m.sor_run(ref, coef, 1.8, 2, n_inner, iters, bct, bcv, 0, s=src)
    return f.download(), ref


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("n,vc,n_inner", [(8, 1, 1), (8, 2, 2), (16, 2, 1), (32, 1, 1)])
def test_sor2_f64_bitexact(gpu_ok, fused, n, vc, n_inner):
    got, ref = run_sor2("f64", n, vc, n_inner, 7, fused)
    assert_bitexact(got, ref, face_mask(n, vc), f"sor2 f64 n={n} vc={vc}")


@pytest.mark.parametrize("n,vc,n_inner", [(8, 1, 1), (8, 2, 2), (16, 2, 1), (32, 1, 1)])
def test_sor2_f32_within_tolerance(gpu_ok, n, vc, n_inner):
    got, ref = run_sor2("f32", n, vc, n_inner, 1, True)
    assert_close_normwise(got, ref, 1e-6, face_mask(n, vc), f"sor2 f32 1 sweep n={n}")
    got, ref = run_sor2("f32", n, vc, n_inner, 10, True)
    assert_close_normwise(got, ref, 1e-5, face_mask(n, vc), f"sor2 f32 10 sweeps n={n}")


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_fused_equals_unfused(gpu_ok, dt):
    a, _ = run_sor2(dt, 16, 2, 1, 9, True, level=3)
    b, _ = run_sor2(dt, 16, 2, 1, 9, False, level=3)
    assert_bitexact(a, b, face_mask(16, 2), f"fused vs unfused {dt}")


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("n,vc", [(8, 2), (16, 1), (16, 2), (32, 1)])
def test_kernel_variants_identical(gpu_ok, dt, n, vc):
    """Every fused kernel shape (one CTA per block with the source in shared
    memory or L1, 256 or 512 threads, persistent bulk-copy pipeline, pull
    form, with the source as is or packed for runs of 8 or more iterations)
    gives the unfused result bit for bit."""
    ref, _ = run_sor2(dt, n, vc, 1, 9, False, level=2)
    for v in range(1, 8):
        got, _ = run_sor2(dt, n, vc, 1, 9, True, level=2, variant=v)
        assert_bitexact(got, ref, face_mask(n, vc), f"variant {v} {dt} n={n} vc={vc}")


def test_autotune_keeps_field_and_picks_a_variant(gpu_ok):
    tree = small_octree(periodic=(False, False, False), level=2, radius=0.3)
    n, vc = 16, 2
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    bct, bcv = outer_dirichlet(tree, 0.0)
    bm.set_boundary(bct, bcv)
    f, s = bm.setDataClass("f32", vc), bm.setDataClass("f32", vc)
    a = np.random.default_rng(2).uniform(size=f.shape).astype(np.float32)
    f.upload(a)
    s.upload(a)
    best, us = bm.autotune_sor(f, bg.sor2_coef(tree.cell_sizes(n)), 1.8, form=2, s=s, iters=3)
    assert 1 <= best <= 7 and us > 0
    assert_bitexact(f.download(), a, what="autotune leaves f unchanged")


def test_sor_f64_n32_in_place_path(gpu_ok):
    """n=32 FP64 does not fit shared memory: the in-place global-memory variant."""
    tree = small_octree(periodic=(True, False, False), level=1, radius=0.3)
    n, vc = 32, 1
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    bct, bcv = outer_dirichlet(tree, 1.0, periodic=(True, False, False))
    bm.set_boundary(bct, bcv, bg.DIRICHLET_BCX)
    f = bm.setDataClass("f64", vc)
    bm.prepareForVCUpdate(f)
    a = np.random.default_rng(5).uniform(size=f.shape)
    f.upload(a)
    coef = bg.sor1_coef(tree.cell_sizes(n), 1.5)
    bm.sor_run(f, coef, 1.5, form=1, n_inner=3, n_outer=4)
    ld, nid, sf, _ = tree.neighbors()
    m = po.OracleMesh(ld, nid, sf, n, vc)
    ref = a.copy()
    m.sor_run(ref, coef, 1.5, 1, 3, 4, bct, bcv, 1)
    assert_bitexact(f.download(), ref, face_mask(n, vc), "sor n=32 f64")
