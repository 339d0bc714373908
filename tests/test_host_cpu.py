"""CPU: the C ABI library loads and exports its header, and the host-side
logic (octree, balancing, orderings, argument checks) behaves -- no kernel is
launched here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import capi
from bcmtools_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    txt = (ROOT / "include" / "bcmg.h").read_text()
    return sorted(set(re.findall(r"BCMG_API\s+[\w\s\*]+?\b(bcmg_\w+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    syms = header_symbols()
    assert len(syms) > 40
    lib = C.CDLL(str(capi.LIB_PATH))
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(capi.EXPORTED), set(syms) ^ set(capi.EXPORTED)


def test_ctypes_signatures_match_header_arity():
    """Every header prototype has a ctypes signature with as many arguments."""
    txt = (ROOT / "include" / "bcmg.h").read_text()
    protos = re.findall(r"BCMG_API\s+[\w\s\*]+?\b(bcmg_\w+)\s*\(([^)]*)\)", txt)
    assert len(protos) == len(header_symbols())
    for name, args in protos:
        a = args.strip()
        n = 0 if a in ("", "void") else len(a.split(","))
        assert len(capi._SIGS[name][1]) == n, name


def test_no_device_is_an_error_code_not_a_crash():
    lib = capi.load()
    ctx = C.c_void_p()
    rc = lib.bcmg_ctx_create(C.byref(ctx), 0)
    if rc == 0:
        lib.bcmg_ctx_destroy(ctx)
        pytest.skip("a GPU is present")
    assert rc == capi.NO_DEVICE


def test_octree_argument_errors():
    lib = capi.load()
    h = C.c_void_p()
    rg = bg.RootGrid(1, 1, 1).to_c()
    d = bg.Divider.flat(16).to_c()  # level beyond the 4-bit pedigree
    assert lib.bcmg_octree_build(C.byref(h), C.byref(rg), C.byref(d), 0, 0) == capi.USAGE
    d = bg.Divider.simple(3, 1).to_c()
    assert lib.bcmg_octree_build(C.byref(h), C.byref(rg), C.byref(d), 0, 0) == capi.USAGE
    assert lib.bcmg_octree_build(None, C.byref(rg), C.byref(d), 0, 0) == capi.USAGE


def test_two_to_one_violation_reported():
    """An unbalanced pedigree list makes neighbors() fail with FAILURE instead of
    exiting (the reference exits, BCMOctree.cpp:462-468)."""
    rg = bg.RootGrid(1, 1, 1)
    peds = []
    for c in range(1, 8):  # level-1 children 1..7
        peds.append(bg.pedigree(1, c & 1, (c >> 1) & 1, (c >> 2) & 1))
    for c in range(8):  # child 0 refined to level 2, one child of it to level 3
        x, y, z = c & 1, (c >> 1) & 1, (c >> 2) & 1
        if c == 1:
            for cc in range(8):
                peds.append(bg.pedigree(3, 2 * x + (cc & 1), 2 * y + ((cc >> 1) & 1),
                                        2 * z + ((cc >> 2) & 1)))
        else:
            peds.append(bg.pedigree(2, x, y, z))
    t = bg.Octree.from_pedigrees(rg, peds)
    with pytest.raises(bg.BcmgError) as e:
        t.neighbors()
    assert e.value.code == capi.FAILURE


def interior_faces_all_have_neighbours(t, periodic):
    ld, nid, sf, outer = t.neighbors()
    has = (nid >= 0).any(axis=2)
    expect = np.ones_like(has)
    for ax in range(3):
        if not periodic[ax]:
            expect[:, 2 * ax:2 * ax + 2] &= outer[:, 2 * ax:2 * ax + 2] == 0
    return np.array_equal(has, expect)


@pytest.mark.parametrize("periodic", [(False, False, False), (True, True, False)])
def test_balanced_tree_is_two_to_one(periodic):
    rg = bg.RootGrid(2, 2, 2, periodic=periodic, root_length=0.5)
    pts = np.array([[0.1, 0.1, 0.1], [0.77, 0.5, 0.33]])
    t = bg.Octree.build(rg, bg.Divider.balls(pts, 0.02, 5), "Z")
    ld, _, _, _ = t.neighbors()
    assert set(np.unique(ld)) <= {-1, 0, 1}
    assert interior_faces_all_have_neighbours(t, periodic)


def test_orderings_permute_the_same_leaves():
    rg = bg.RootGrid(2, 1, 1, periodic=(True, False, False), root_length=0.5)
    div = bg.Divider.sphere_surface((0.5, 0.25, 0.25), 0.2, 3)
    tz = bg.Octree.build(rg, div, "Z")
    for ordering in ("HILBERT", "RANDOM"):
        t = bg.Octree.build(rg, div, ordering, seed=5)
        assert sorted(t.pedigrees.tolist()) == sorted(tz.pedigrees.tolist())
        # neighbour tables agree after mapping ids through the permutation
        pos = {p: i for i, p in enumerate(tz.pedigrees.tolist())}
        perm = np.array([pos[p] for p in t.pedigrees.tolist()])
        ld, nid, sf, _ = t.neighbors()
        ldz, nidz, sfz, _ = tz.neighbors()
        assert np.array_equal(ldz[perm], ld) and np.array_equal(sfz[perm], sf)
        mapped = np.where(nid >= 0, perm[np.maximum(nid, 0)], -1)
        assert np.array_equal(nidz[perm], mapped)


def test_pedigree_roundtrip():
    w = W.two_level_sphere(n=16, vc=2)
    t2 = bg.Octree.from_pedigrees(w.tree.rootgrid, w.tree.pedigrees)
    a, b = w.tree.neighbors(), t2.neighbors()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_benchmark_mesh_sizes():
    assert W.plain_poisson().nb == 512
    w2 = W.two_level_sphere()
    assert 3000 <= w2.nb <= 5000 and set(np.bincount(w2.tree.levels).nonzero()[0]) == {0, 1, 2, 3}
    ld, _, _, _ = w2.neighbors()
    assert set(np.unique(ld)) == {-1, 0, 1}
    w3 = W.points_level5()
    assert 2000 <= w3.nb <= 6000 and w3.n == 32 and w3.tree.levels.max() == 5


def test_random_instances_are_seeded():
    a = W.random_instance(1000)
    b = W.random_instance(1000)
    assert np.array_equal(a.tree.pedigrees, b.tree.pedigrees) and a.n == b.n
    assert 32 <= a.nb <= 6000


def test_layout_info_matches_the_sor1_log():
    """printBlockLayoutInfo's counts for sor1's mesh (rebuilt here from the
    reference's pedigree list) against the reference's shipped log
    (examples/sor1/log.4:25-47: 8 + 448 blocks; faces summed over its four
    ranks' intra- and inter-node counts: 16+80, 618+1870, 16+80)."""
    from bcmtools_gb300.mesh import Partition, format_layout_info, layout_info
    g = np.load(ROOT / "tests" / "golden" / "sor1.npz")
    rg = bg.RootGrid(1, 1, 1, periodic=(False, True, True))
    t = bg.Octree.from_pedigrees(rg, g["pedigrees"])
    ld, nid, _, _ = t.neighbors()
    info = layout_info(t.levels, ld, nid)
    assert (info["level_min"], info["level_max"]) == (2, 3)
    assert info["blocks"] == {2: 8, 3: 448} and info["total"] == 456
    assert info["faces_intra"] == [16 + 80, 618 + 1870, 16 + 80]
    assert info["faces_inter"] == [0, 0, 0]
    part = Partition(4, 456)  # log.4:20-23: [0:113] [114:227] [228:341] [342:455]
    assert [(part.getStart(r), part.getEnd(r) - 1) for r in range(4)] == \
        [(0, 113), (114, 227), (228, 341), (342, 455)]
    split = layout_info(t.levels, ld, nid, ranks=part.ranks())
    assert [a + b for a, b in zip(split["faces_intra"], split["faces_inter"])] == \
        info["faces_intra"]
    txt = format_layout_info(info)
    assert "    L=3: 448" in txt and "        dLevel= 0: 2488" in txt


def test_partition_matches_reference_rule():
    """Partition.h:46-58: the first n % p ranks take one more item."""
    from bcmtools_gb300.mesh import Partition
    p = Partition(4, 10)
    assert [p.getNum(r) for r in range(4)] == [3, 3, 2, 2]
    assert [p.getRank(i) for i in range(-1, 11)] == [-1, 0, 0, 0, 1, 1, 1, 2, 2, 3, 3, -1]
    assert list(p.ranks()) == [0, 0, 0, 1, 1, 1, 2, 2, 3, 3]
    assert Partition(4, 996).getNum(3) == 249  # ParametricDivider/log_sphere.4:15-19


def inter_faces_per_rank(ld, nid, rk, nranks):
    """Inter-node faces of every rank: faces of its blocks whose neighbour
    (per subface at level difference +1) lives on another rank."""
    out = []
    for r in range(nranks):
        mine = rk == r
        cnt = 0
        for d in (-1, 0, 1):
            nsub = 4 if d == 1 else 1
            sel = (ld == d)[:, :, None] & (nid[:, :, :nsub] >= 0) & mine[:, None, None]
            cnt += int((rk[nid[:, :, :nsub][sel]] != r).sum())
        out.append(cnt)
    return out


def test_layout_matches_the_cylinder_log():
    """examples/ParametricDivider/log_cylinder.4:4-47 (root grid 1x1x2,
    levels 0..4, axis (0.5, 0.5), r = 0.4, Hilbert, four ranks)."""
    from bcmtools_gb300.mesh import Partition, layout_info
    t = bg.Octree.build(bg.RootGrid(1, 1, 2), bg.Divider.cylinder((0.5, 0.5), 0.4, 0, 4),
                        "HILBERT")
    ld, nid, _, _ = t.neighbors()
    part = Partition(4, t.num_leaves)
    info = layout_info(t.levels, ld, nid, ranks=part.ranks())
    assert (info["level_min"], info["level_max"]) == (3, 4)
    assert info["blocks"] == {3: 384, 4: 1920} and info["total"] == 2304
    assert info["faces_intra"] == [1536, 9440, 1536]
    assert info["faces_inter"] == [0, 504, 0]
    inter = inter_faces_per_rank(ld, nid, part.ranks(), 4)
    assert (min(inter), max(inter), sum(inter) / 4) == (84, 168, 126.0)


def test_layout_matches_the_sphere_log():
    """The sphere layout of examples/ParametricDivider/log_sphere.4:4-49
    (root grid 2x1x1, levels 0..4, c = (0.8, 0.5, 0.5), r = 0.25, Hilbert,
    four ranks), rebuilt here with the extra margin ratio 1e-6 of main.cpp's
    alternative divider call: every count of the log, intra- and inter-node."""
    from bcmtools_gb300.mesh import Partition, layout_info
    t = bg.Octree.build(bg.RootGrid(2, 1, 1),
                        bg.Divider.sphere((0.8, 0.5, 0.5), 0.25, 0, 4, margin_ratio=1e-6),
                        "HILBERT")
    ld, nid, _, _ = t.neighbors()
    part = Partition(4, t.num_leaves)
    info = layout_info(t.levels, ld, nid, ranks=part.ranks())
    assert (info["level_min"], info["level_max"]) == (1, 4)
    assert info["blocks"] == {1: 4, 2: 32, 3: 428, 4: 532} and info["total"] == 996
    assert info["faces_intra"] == [546, 4098, 546]
    assert info["faces_inter"] == [142, 510, 142]
    inter = inter_faces_per_rank(ld, nid, part.ranks(), 4)
    assert (min(inter), max(inter), sum(inter) / 4) == (141, 244, 198.5)


def test_device_mesh_attributes_match_the_host_octree():
    """DeviceMesh (the device set-up's mesh read back) derives levels,
    origins and block sizes from the pedigrees as the host octree reports
    them, on a root grid with an origin, a root length and several roots."""
    from bcmtools_gb300.mesh import DeviceMesh
    rg = bg.RootGrid(3, 2, 1, periodic=(False, True, False), origin=(1.0, -2.0, 0.5),
                     root_length=2.0)
    t = bg.Octree.build(rg, bg.Divider.balls([[2.0, -1.0, 1.5], [4.5, 0.5, 1.0]], 0.2, 4,
                                             min_level=1), "Z")
    ld, nid, sf, outer = t.neighbors()
    m = DeviceMesh(rg, t.pedigrees, ld, nid, sf, outer)
    assert m.num_leaves == t.num_leaves
    assert np.array_equal(m.levels, t.levels)
    assert np.allclose(m.origins, t.origins, rtol=0, atol=1e-12)
    assert np.allclose(m.block_sizes, t.block_sizes, rtol=0, atol=0)
    assert np.array_equal(m.cell_sizes(16), t.cell_sizes(16))
    for a, b in zip(m.neighbors(), t.neighbors()):
        assert np.array_equal(a, b)
