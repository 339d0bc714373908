"""CPU: pin the oracle and the octree builder to the reference's own outputs.

The golden fixtures were produced by the reference library compiled from its
sources (tests/golden/make_golden.py): BCMOctree neighbour tables,
BlockManager::updateVC through Scalar3DUpdater<T> (real_type float and
double), the examples/sor1 run whose errorMax is the reference's shipped
known answer (examples/sor1/log.4:54), and the examples/sor2 run (RB-SOR with
a source term) on its shipped test.conf.
"""
import hashlib
import math

import numpy as np
import pytest

import bcmtools_gb300 as bg
from oracle import pyoracle as po
from tests.helpers import GOLDEN, assert_bitexact, face_mask, splitmix_uniform

TREES = {
    "tree_simple03_pyz": (bg.RootGrid(1, 1, 1, (False, True, True)), bg.Divider.simple(0, 3)),
    "tree_simple13_2x1x1": (bg.RootGrid(2, 1, 1), bg.Divider.simple(1, 3)),
    "tree_flat2_px": (bg.RootGrid(1, 2, 1, (True, False, False)), bg.Divider.flat(2)),
}


@pytest.mark.parametrize("name", sorted(TREES))
def test_octree_matches_reference(name):
    g = np.load(GOLDEN / f"{name}.npz")
    rg, div = TREES[name]
    div.balance = False  # the reference does not balance; these trees are 2:1 already
    t = bg.Octree.build(rg, div, "Z")
    ld, nid, sf, _ = t.neighbors()
    assert t.num_leaves == int(g["nb"])
    assert np.array_equal(t.pedigrees, g["pedigrees"])
    assert np.array_equal(ld, g["ld"])
    assert np.array_equal(nid, g["id"])
    assert np.array_equal(sf, g["sf"])
    assert np.allclose(t.origins, g["origins"], rtol=0, atol=1e-15)


def test_sphere_octree_matches_reference():
    """SphereDivider (inactive interior, ripple margin, float arithmetic) in
    the reference's Hilbert order: the same leaves, order and neighbour
    tables as the reference-built tree of log_sphere.4's configuration."""
    g = np.load(GOLDEN / "tree_sphere_2x1x1.npz")
    t = bg.Octree.build(bg.RootGrid(2, 1, 1),
                        bg.Divider.sphere((0.8, 0.5, 0.5), 0.25, 0, 4, margin_ratio=1e-6),
                        "HILBERT")
    ld, nid, sf, _ = t.neighbors()
    assert t.num_leaves == int(g["nb"]) == 996
    assert np.array_equal(t.pedigrees, g["pedigrees"])
    assert np.array_equal(ld, g["ld"]) and np.array_equal(nid, g["id"])
    assert np.array_equal(sf, g["sf"])


def test_cylinder_octree_matches_reference():
    """CylinderDivider (blocks outside the cylinder inactive) in Hilbert order:
    the reference-built tree of log_cylinder.4's configuration."""
    g = np.load(GOLDEN / "tree_cylinder_1x1x2.npz")
    t = bg.Octree.build(bg.RootGrid(1, 1, 2), bg.Divider.cylinder((0.5, 0.5), 0.4, 0, 4),
                        "HILBERT")
    ld, nid, sf, _ = t.neighbors()
    assert t.num_leaves == int(g["nb"]) == 2304
    assert np.array_equal(t.pedigrees, g["pedigrees"])
    assert np.array_equal(ld, g["ld"]) and np.array_equal(nid, g["id"])
    assert np.array_equal(sf, g["sf"])


@pytest.mark.parametrize("origin,length", [((0.0, 0.0, 0.0), 2.0), ((-1.0, 0.0, 0.0), 1.0),
                                           ((0.5, -3.0, 2.0), 0.125)])
def test_sphere_cylinder_ignore_root_frame(origin, length):
    """The reference builds SphereDivider and CylinderDivider over origin 0
    and root length 1 (SphereDivider.h:72, CylinderDivider.h:69), so their
    trees depend only on the root index grid: a mesh with another origin or
    root length gives the reference-built trees all the same."""
    gs = np.load(GOLDEN / "tree_sphere_2x1x1.npz")
    t = bg.Octree.build(bg.RootGrid(2, 1, 1, origin=origin, root_length=length),
                        bg.Divider.sphere((0.8, 0.5, 0.5), 0.25, 0, 4, margin_ratio=1e-6),
                        "HILBERT")
    assert t.num_leaves == 996 and np.array_equal(t.pedigrees, gs["pedigrees"])
    gc = np.load(GOLDEN / "tree_cylinder_1x1x2.npz")
    t = bg.Octree.build(bg.RootGrid(1, 1, 2, origin=origin, root_length=length),
                        bg.Divider.cylinder((0.5, 0.5), 0.4, 0, 4), "HILBERT")
    assert t.num_leaves == 2304 and np.array_equal(t.pedigrees, gc["pedigrees"])


def test_hilbert_order_matches_reference():
    """sor2's mesh (SimpleDivider 0..3, examples/sor2/test.conf) built here in
    Hilbert order lists its leaves in the reference run's order."""
    g = np.load(GOLDEN / "sor2.npz")
    div = bg.Divider.simple(0, 3)
    div.balance = False
    t = bg.Octree.build(bg.RootGrid(1, 1, 1), div, "HILBERT")
    assert np.array_equal(t.pedigrees, g["pedigrees"])


def test_octree_from_reference_pedigrees():
    """The VC fixture mesh's reference neighbour tables from its pedigree list."""
    g = np.load(GOLDEN / "vc_f64_n4_vc1.npz")
    rg = bg.RootGrid(2, 2, 2, periodic=(True, False, False), root_length=0.5)
    t = bg.Octree.from_pedigrees(rg, g["pedigrees"])
    ld, nid, sf, _ = t.neighbors()
    assert np.array_equal(ld, g["ld"]) and np.array_equal(nid, g["id"])
    assert np.array_equal(sf, g["sf"])
    assert set(np.unique(ld)) == {-1, 0, 1}


VC_CASES = ["vc_f32_n4_vc1", "vc_f32_n4_vc2", "vc_f64_n4_vc1", "vc_f64_n4_vc2"]


def vc_case(name):
    g = np.load(GOLDEN / f"{name}.npz")
    dt = np.float32 if "f32" in name else np.float64
    n, vc = int(g["n"]), int(g["vc"])
    m = po.OracleMesh(g["ld"], g["id"], g["sf"], n, vc)
    a = splitmix_uniform(int(g["seed"]), m.nb * m.brick).astype(dt).reshape(m.shape)
    return g, m, a


@pytest.mark.parametrize("name", VC_CASES)
def test_oracle_vc_update_bitexact(name):
    g, m, a = vc_case(name)
    m.vc_update(a)
    assert_bitexact(a, g["after"], what=name)


@pytest.mark.parametrize("name", VC_CASES)
def test_oracle_separate_updates_compose(name):
    """SeparateXYZ and SeparateXYZ_SeparateLevelDiff orders give the AtOnce result
    (reads are interior-only, writes disjoint ghost slabs)."""
    g, m, a = vc_case(name)
    b = a.copy()
    for ax in range(3):
        m.vc_update(a, 1 << ax, 7)
    for ldbit in (4, 2, 1):  # F2C, flat, C2F (LocalScalar3D.h:214-224)
        for ax in range(3):
            m.vc_update(b, 1 << ax, ldbit)
    assert_bitexact(a, g["after"], what=name + " xyz")
    assert_bitexact(b, g["after"], what=name + " xyz+ld")


VCD_CASES = ["vcd_f32_n8_vc3", "vcd_f64_n8_vc3", "vcd_f32_n16_vc2", "vcd_f64_n16_vc2"]


def ghost_digest(field, n, vc):
    sel = np.ascontiguousarray(field[:, face_mask(n, vc)])
    return hashlib.sha256(sel.astype(sel.dtype.newbyteorder("<")).tobytes()).hexdigest()


@pytest.mark.parametrize("name", VCD_CASES)
def test_oracle_vc_update_matches_reference_digest(name):
    """updateVC at 8 cells / vc = 3 and 16 cells / vc = 2: the sampled blocks
    cell by cell and the whole result by SHA-256 against the reference's."""
    g = np.load(GOLDEN / f"{name}.npz")
    dt = np.float32 if "f32" in name else np.float64
    n, vc = int(g["n"]), int(g["vc"])
    m = po.OracleMesh(g["ld"], g["id"], g["sf"], n, vc)
    a = splitmix_uniform(int(g["seed"]), int(np.prod(m.shape))).astype(dt).reshape(m.shape)
    m.vc_update(a)
    assert_bitexact(a[g["sample_blocks"]], g["sample_after"], face_mask(n, vc), name)
    assert ghost_digest(a, n, vc) == str(g["digest"])


def sor1_setup():
    g = np.load(GOLDEN / "sor1.npz")
    n, vc = int(g["n"]), int(g["vc"])
    bct = np.where(g["bc_type"] == 1, 1, 0).astype(np.int32)  # BoundaryInfo::DIRICHLET
    bcv = np.where(g["bc_id"] == 1, float(g["b1"]), float(g["b0"]))
    coef = bg.sor1_coef(g["cell_sizes"], float(g["omega"]))
    return g, n, vc, bct, bcv, coef


def test_oracle_sor1_known_answer():
    """sor1 on its shipped test.conf: field identical to the reference run and
    errorMax = 0.00353051 (examples/sor1/log.4:54)."""
    g, n, vc, bct, bcv, coef = sor1_setup()
    m = po.OracleMesh(g["ld"], g["id"], g["sf"], n, vc)
    f = np.zeros(m.shape)
    m.vc_update(f)
    m.dirichlet(f, bct, bcv, 0)
    m.sor_run(f, coef, float(g["omega"]), 1, int(g["n_inner"]), int(g["n_outer"]), bct, bcv, 0)
    assert_bitexact(f, g["field"], face_mask(n, vc), "sor1")
    xs = g["origins"][:, 0, None] + (np.arange(n) + 0.5)[None, :] * g["cell_sizes"][:, 0, None]
    err = np.abs(f[:, vc:-vc, vc:-vc, vc:-vc] - xs[:, None, None, :]).max()
    assert f"{err:.6g}" == "0.00353051"
    assert str(g["error_max_line"]).endswith("0.00353051")


def test_oracle_sor2_matches_reference_run():
    """sor2 (RB-SOR with a source term, examples/sor2/Solver.cpp:77-160) on its
    shipped test.conf -- 456 blocks of levels 0..3 in Hilbert order, 400 outer
    iterations at omega 1.4 -- gives the reference run's field bit for bit:
    the sampled blocks compared cell by cell, the whole field by SHA-256."""
    g = np.load(GOLDEN / "sor2.npz")
    n, vc = int(g["n"]), int(g["vc"])
    nb = g["ld"].shape[0]
    m = po.OracleMesh(g["ld"], g["id"], g["sf"], n, vc)
    a = 2 * math.pi
    cc = -3.0 * a * a
    s = np.zeros(m.shape)
    for b in range(nb):
        sx, sy, sz = g["source_factors"][b]
        # ((c sx) sy) sz, the reference's operation order (Solver.cpp:401)
        s[b, vc:-vc, vc:-vc, vc:-vc] = ((cc * sx[None, None, :]) * sy[None, :, None]) * \
            sz[:, None, None]
    bct = np.where(g["bc_type"] == 1, 1, 0).astype(np.int32)  # BoundaryInfo::DIRICHLET
    bcv = np.zeros((nb, 6))  # sor2/main.cpp:133-134
    f = np.zeros(m.shape)
    m.vc_update(f)
    m.dirichlet(f, bct, bcv, 0)
    m.sor_run(f, bg.sor2_coef(g["cell_sizes"]), float(g["omega"]), 2, int(g["n_inner"]),
              int(g["n_outer"]), bct, bcv, 0, s=s)
    assert_bitexact(f[g["sample_blocks"]], g["sample_field"], face_mask(n, vc), "sor2 sample")
    assert ghost_digest(f, n, vc) == str(g["field_sha256"])


def test_oracle_planted_mistake_is_caught():
    """A mistake planted in the oracle's input (one wrong neighbour subface)
    changes the result, so the bit-exact check has teeth."""
    g, m, a = vc_case("vc_f64_n4_vc1")
    sf = g["sf"].copy()
    ld = g["ld"]
    k = np.argwhere(ld == -1)[0]
    sf[k[0], k[1]] = (sf[k[0], k[1]] + 1) % 4
    bad = po.OracleMesh(g["ld"], g["id"], sf, int(g["n"]), int(g["vc"]))
    b = a.copy()
    bad.vc_update(b)
    with pytest.raises(AssertionError):
        assert_bitexact(b, g["after"], what="planted")
