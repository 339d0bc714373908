"""GPU: the device-side mesh set-up against the host octree builder.

The octree of a divider built level by level on the GPU, its 2:1 balance,
the Z order of its leaves and the neighbour table (BCMOctree.cpp:23-41,
66-96, 423-478) must equal what the host builder gives (octree.cpp, itself
checked against the reference's layouts and golden ghost updates): the same
leaves in the same order and the same level differences, neighbour ids,
subfaces and outer flags, for every divider kind and for pedigree lists in
any order.  Registering through the device set-up must then solve bit for
bit as registering the host tables does.
"""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from bcmtools_gb300 import capi
from bcmtools_gb300 import workloads as W
from oracle import pyoracle as po
from tests.helpers import assert_bitexact, face_mask

pytestmark = pytest.mark.gpu

RG1 = bg.RootGrid(1, 1, 1)
RG2P = bg.RootGrid(2, 2, 2, periodic=(True, False, True), root_length=0.5)
RG4 = bg.RootGrid(4, 4, 4, root_length=0.25)
RG32 = bg.RootGrid(3, 2, 1, periodic=(False, True, False), origin=(1.0, -2.0, 0.5),
                   root_length=2.0)

CASES = {
    "flat3": (RG1, bg.Divider.flat(3)),
    "flat2_rg4": (RG4, bg.Divider.flat(2)),
    "simple": (RG32, bg.Divider.simple(1, 4, 0)),
    "simple_x": (RG2P, bg.Divider.simple(0, 3, 3)),
    "surface": (RG4, bg.Divider.sphere_surface((0.5, 0.5, 0.5), 0.3, 3)),
    "surface_p": (RG2P, bg.Divider.sphere_surface((0.5, 0.5, 0.5), 0.32, 4, min_level=1)),
    "balls": (RG1, bg.Divider.balls(np.random.default_rng(3).uniform(0, 1, (16, 3)), 0.05, 5)),
    "balls_rg32": (RG32, bg.Divider.balls([[2.0, -1.0, 1.5], [4.5, 0.5, 1.0]], 0.2, 5,
                                          min_level=1)),
    "sphere": (bg.RootGrid(2, 2, 2), bg.Divider.sphere((1.0, 1.0, 1.0), 0.6, 1, 4)),
    "cylinder": (bg.RootGrid(2, 2, 1), bg.Divider.cylinder((1.0, 1.0), 0.7, 1, 4)),
}


def _unbalanced(div):
    d = bg.Divider(**{k: v for k, v in div.__dict__.items() if k != "_keep"})
    d.balance = False
    return d


def host_tables(rg, div):
    t = bg.Octree.build(rg, div, "Z")
    try:
        return t, t.neighbors()
    except capi.BcmgError as e:
        return t, e


def device_tables(rg, div, n=8):
    bm = bg.BlockManager(0)
    try:
        m = bm.build_mesh(rg, div, n)
        return bm, m, m.neighbors()
    except capi.BcmgError as e:
        return bm, None, e


def assert_same_tables(host, dev, what):
    for name, a, b in zip(("ld", "id", "sf", "outer"), host, dev):
        assert np.array_equal(a, b), f"{what}: {name} differs at {np.argwhere(a != b)[:5]}"


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_build_equals_host_build(gpu_ok, name):
    rg, div = CASES[name]
    tree, ht = host_tables(rg, div)
    bm, m, dt = device_tables(rg, div)
    if isinstance(ht, Exception):
        # a tree the host cannot describe (a face across two levels) fails alike
        assert isinstance(dt, capi.BcmgError) and dt.code == capi.FAILURE, name
        return
    assert m is not None, dt
    assert m.num_leaves == tree.num_leaves
    assert np.array_equal(m.pedigrees, tree.pedigrees), name
    assert_same_tables(ht, dt, name)
    assert np.allclose(m.origins, tree.origins) and np.allclose(m.block_sizes, tree.block_sizes)


@pytest.mark.parametrize("name", ["surface", "balls", "balls_rg32", "surface_p"])
def test_device_balance_of_a_pedigree_list(gpu_ok, name):
    """The unbalanced tree's leaves, shuffled, balanced on the device: the
    host's balanced tree, leaves in Z order."""
    rg, div = CASES[name]
    loose = bg.Octree.build(rg, _unbalanced(div), "Z")
    peds = np.random.default_rng(7).permutation(loose.pedigrees)
    tight = bg.Octree.build(rg, div, "Z")
    bm = bg.BlockManager(0)
    m = bm.register_pedigrees(rg, peds, 8, balance=True)
    assert np.array_equal(m.pedigrees, tight.pedigrees), name
    assert_same_tables(tight.neighbors(), m.neighbors(), name)


@pytest.mark.parametrize("name", ["surface", "balls", "sphere", "simple"])
def test_device_neighbours_of_a_pedigree_list(gpu_ok, name):
    """Leaves in a random order (blocks in that order), with some of them left
    out (their regions inactive): the host's from_pedigrees tables."""
    rg, div = CASES[name]
    t = bg.Octree.build(rg, div, "Z")
    rng = np.random.default_rng(11)
    peds = rng.permutation(t.pedigrees)
    peds = peds[rng.uniform(size=len(peds)) > 0.1]
    host = bg.Octree.from_pedigrees(rg, peds)
    try:
        ht = host.neighbors()
    except capi.BcmgError:
        pytest.skip("the reduced list is not 2:1 balanced")
    bm = bg.BlockManager(0)
    m = bm.register_pedigrees(rg, peds, 8)
    assert np.array_equal(m.pedigrees, peds)
    assert_same_tables(ht, m.neighbors(), name)


def test_device_pedigree_list_errors(gpu_ok):
    t = bg.Octree.build(RG1, bg.Divider.flat(2), "Z")
    peds = t.pedigrees
    for bad in (np.concatenate([peds, peds[:1]]),  # listed twice
                np.concatenate([peds, [bg.mesh.pedigree(1, 0, 0, 0)]])):  # above other leaves
        bm = bg.BlockManager(0)
        with pytest.raises(capi.BcmgError) as e:
            bm.register_pedigrees(RG1, bad, 8)
        assert e.value.code == capi.USAGE
    # a face spanning two levels (unbalanced, and no balancing asked for)
    loose = bg.Octree.build(RG1, _unbalanced(CASES["balls"][1]), "Z")
    with pytest.raises(capi.BcmgError):
        loose.neighbors()
    bm = bg.BlockManager(0)
    with pytest.raises(capi.BcmgError) as e:
        bm.register_pedigrees(RG1, loose.pedigrees, 8)
    assert e.value.code == capi.FAILURE


def test_device_batch_equals_meshes_alone(gpu_ok):
    specs = [CASES["balls"], CASES["surface"], (RG1, bg.Divider.flat(1)), CASES["balls_rg32"]]
    bm = bg.BlockManager(0)
    first, meshes = bm.build_mesh_batch(specs, 8)
    sizes = []
    for (rg, div), m in zip(specs, meshes):
        tree, ht = host_tables(rg, div)
        assert np.array_equal(m.pedigrees, tree.pedigrees)
        assert_same_tables(ht, m.neighbors(), "batch")
        sizes.append(tree.num_leaves)
    assert first == list(np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert bm.nb == sum(sizes)


def test_c2_sor_on_the_device_mesh_bitexact(gpu_ok):
    """The two-level sphere mesh (4432 blocks of 16^3, vc = 2) registered by
    the device set-up: 10 FP64 red-black SOR iterations equal the oracle's on
    the host tree bit for bit (the fused pull-form kernel with the face
    tables the device built)."""
    w = W.two_level_sphere(n=16, vc=2)
    bm = bg.BlockManager(0)
    m = bm.build_mesh(w.tree.rootgrid, bg.Divider.sphere_surface((0.5, 0.5, 0.5), 0.3, 3), w.n)
    assert np.array_equal(m.pedigrees, w.tree.pedigrees)
    bct, bcv = w.dirichlet(0.0)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    coef = bg.sor2_coef(m.cell_sizes(w.n))
    f, s = bm.setDataClass("f64", w.vc), bm.setDataClass("f64", w.vc)
    bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
    s_host = W.rhs_gaussian(w, seed=2, dtype=np.float64)
    s.upload(s_host)
    f.fill(0.0)
    bm.imposeBoundaryCondition(f)
    bm.sor_run(f, coef, 1.8, form=2, n_inner=1, n_outer=10, s=s)
    got = f.download()
    ld, nid, sf, _ = w.neighbors()
    om = po.OracleMesh(ld, nid, sf, w.n, w.vc)
    ref = np.zeros(om.shape)
    om.vc_update(ref)
    om.dirichlet(ref, bct, bcv, 0)
    om.sor_run(ref, coef, 1.8, 2, 1, 10, bct, bcv, 0, s=s_host)
    assert_bitexact(got, ref, face_mask(w.n, w.vc), "C2 SOR f64 on the device mesh")


def test_device_mesh_solve_equals_host_registration(gpu_ok):
    """A balls mesh of 16^3 blocks: mixed-precision BiCGSTAB through the
    device set-up and through the host tables -- same iterations, same field."""
    rg, div = CASES["balls"]
    out = []
    for dev in (False, True):
        bm = bg.BlockManager(0)
        if dev:
            tree = bm.build_mesh(rg, div, 16)
            outer = tree.neighbors()[3]
        else:
            tree = bg.Octree.build(rg, div, "Z")
            outer = bm.register_octree(tree, 16)
        t = (outer != 0).astype(np.int32)
        bm.set_boundary(t, np.zeros(t.shape), bg.DIRICHLET_SOR)
        op = bm.op_const(bg.laplace_coef(tree.cell_sizes(16)))
        x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
        b.fill(0.0)
        b.fill_random(4)
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        info = bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=60, eps_inner=1e-2,
                                 max_outer=20, eps=1e-9)
        out.append((info.iterations, info.refinements, x.download()))
        bm.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
