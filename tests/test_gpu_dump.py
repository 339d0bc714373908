"""GPU: checkpoint / restart of a field in the per-block dump format of
SolverTest's LocalScalar3D::Dump / Load: ghosts imposed before the dump and
after the load; a restart on blocks with twice the cells per axis injects."""
import numpy as np
import pytest

import bcmtools_gb300 as bg
from tests.helpers import outer_dirichlet, small_octree

pytestmark = pytest.mark.gpu


def make(tree, n, vc, dt="f32"):
    bm = bg.BlockManager(0)
    bm.register_octree(tree, n)
    bct, bcv = outer_dirichlet(tree, 0.5)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    f = bm.setDataClass(dt, vc)
    bm.prepareForVCUpdate(f)
    return bm, f


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_dump_then_load_gives_the_field_back(gpu_ok, tmp_path, dt):
    tree = small_octree(level=2, radius=0.3)
    bm, f = make(tree, 8, 2, dt)
    f.fill_random(11)
    f.dump(7, "phi", str(tmp_path))
    want = f.download()  # ghosts imposed by the dump
    _, g = make(tree, 8, 2, dt)
    g.load(7, "phi", str(tmp_path))
    assert np.array_equal(g.download(), want)


def test_restart_on_blocks_with_twice_the_cells(gpu_ok, tmp_path):
    tree = small_octree(level=2, radius=0.3)
    _, coarse = make(tree, 4, 1)
    coarse.fill_random(5)
    coarse.dump(0, "u", str(tmp_path))
    c = coarse.download()
    bm, fine = make(tree, 8, 1)
    fine.load(0, "u", str(tmp_path))
    got = fine.download()
    inj = c[:, 1:-1, 1:-1, 1:-1].repeat(2, 1).repeat(2, 2).repeat(2, 3)
    assert np.array_equal(got[:, 1:-1, 1:-1, 1:-1], inj)
    # ghosts: the boundary conditions and ghost update of the injected field
    _, ref = make(tree, 8, 1)
    a = ref.download()
    a[:, 1:-1, 1:-1, 1:-1] = inj
    ref.upload(a)
    ref.bm.imposeBoundaryCondition(ref)
    r = ref.download()
    mask = np.ones(r.shape[1:], bool)
    mask[0, 0, :] = mask[0, -1, :] = mask[-1, 0, :] = mask[-1, -1, :] = False
    mask[:, 0, 0] = mask[:, 0, -1] = mask[:, -1, 0] = mask[:, -1, -1] = False
    mask[0, :, 0] = mask[0, :, -1] = mask[-1, :, 0] = mask[-1, :, -1] = False
    assert np.array_equal(got[:, mask], r[:, mask])
