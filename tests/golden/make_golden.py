"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference sources (read-only) and a C++
compiler:

    make -C oracle ref          # builds oracle/_ref/{refvc_f,refvc_d,refsor1,refsor2}
    python tests/golden/make_golden.py

The drivers in oracle/_ref/ are the reference library's own BCMOctree,
BlockManager, Scalar3DUpdater<T> and examples/sor1, sor2 Solvers compiled from its
sources (see oracle/Makefile); this script only feeds them inputs and packs
their outputs.  Fixtures:

  tree_*.npz   leaves and NeighborInfo tables of reference-built octrees
               (Flat / Simple dividers in Z order; Sphere- and CylinderDivider
               in Hilbert order with inactive leaves, the layouts of
               log_sphere.4 and log_cylinder.4)
  vc_*.npz     one BlockManager::updateVC of a seeded field on a mesh with
               all three level differences (inputs regenerate from the seed)
  vcd_*.npz    the same at 8 cells / vc = 3 and 16 cells / vc = 2, stored as a
               SHA-256 of the result plus a sample of whole blocks
  sor1.npz     examples/sor1 on its shipped test.conf: final field, whose
               errorMax is the reference's known answer 0.00353051
  sor2.npz     examples/sor2 (RB-SOR with a source term) on its shipped
               test.conf: the source factors, a SHA-256 of the final field
               (interior and face ghosts) and the full field of a sample of
               blocks -- the whole field would be megabytes
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("BCMTOOLS_REF", "/root/reference"))
DRV = ROOT / "oracle" / "_ref"
sys.path.insert(0, str(ROOT))


def splitmix_uniform(seed: int, n: int) -> np.ndarray:
    """The seeded fill of oracle/refvc.cpp: splitmix64 -> uniform [-1, 1) doubles."""
    golden = np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        s = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * golden
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def read_blocks(buf: bytes, with_bc: bool = False):
    off = 0

    def take(dt, cnt):
        nonlocal off
        a = np.frombuffer(buf, dtype=dt, count=cnt, offset=off)
        off += a.nbytes
        return a

    hdr = take(np.int32, 3 if with_bc else 4)
    nb = int(hdr[0])
    peds = np.zeros(nb, np.uint64)
    lev = np.zeros(nb, np.int32)
    org = np.zeros((nb, 3))
    bsz = np.zeros((nb, 3))
    bct = np.zeros((nb, 6), np.int32)
    bci = np.zeros((nb, 6), np.int32)
    ld = np.zeros((nb, 6), np.int32)
    nid = np.zeros((nb, 6, 4), np.int32)
    sf = np.zeros((nb, 6), np.int32)
    for b in range(nb):
        peds[b] = take(np.uint64, 1)[0]
        lev[b] = take(np.int32, 1)[0]
        org[b] = take(np.float64, 3)
        bsz[b] = take(np.float64, 3)
        if with_bc:
            bct[b] = take(np.int32, 6)
            bci[b] = take(np.int32, 6)
        rec = take(np.int32, 36).reshape(6, 6)
        ld[b], nid[b], sf[b] = rec[:, 0], rec[:, 1:5], rec[:, 5]
    out = dict(nb=nb, hdr=hdr, pedigrees=peds, levels=lev, origins=org, sizes=bsz,
               ld=ld, id=nid, sf=sf)
    if with_bc:
        out.update(bc_type=bct, bc_id=bci)
    return out, off


def gen_trees():
    cases = {
        "tree_simple03_pyz": ("1 1 1 6 simple 0 3 Z 2"),
        "tree_simple13_2x1x1": ("2 1 1 0 simple 1 3 Z 4"),
        "tree_flat2_px": ("1 2 1 1 flat 0 2 Z 4"),
    }
    for name, args in cases.items():
        with tempfile.TemporaryDirectory() as td:
            out = Path(td) / "t.bin"
            subprocess.run([str(DRV / "refvc_d"), "tree", *args.split(), str(out)], check=True)
            d, _ = read_blocks(out.read_bytes())
        a = args.split()
        np.savez_compressed(HERE / f"{name}.npz", root=np.array([int(x) for x in a[:4]]),
                            kind=a[4], min_level=int(a[5]), max_level=int(a[6]),
                            **{k: v for k, v in d.items() if k not in ("hdr",)})
        print(name, d["nb"], "blocks")


def gen_sphere_tree():
    """The reference's SphereDivider (float build) on the configuration of
    examples/ParametricDivider/log_sphere.4: root grid 2x1x1, levels 0..4,
    sphere c = (0.8, 0.5, 0.5), r = 0.25, extra margin ratio 1e-6, Hilbert."""
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "t.bin"
        subprocess.run([str(DRV / "refvc_f"), "tree", "2", "1", "1", "0",
                        "sphere:0.8,0.5,0.5,0.25,1e-6", "0", "4", "H", "2", str(out)], check=True)
        d, _ = read_blocks(out.read_bytes())
    np.savez_compressed(HERE / "tree_sphere_2x1x1.npz", nb=d["nb"], pedigrees=d["pedigrees"],
                        levels=d["levels"], ld=d["ld"], id=d["id"], sf=d["sf"],
                        origins=d["origins"])
    print("tree_sphere_2x1x1", d["nb"], "blocks")


def gen_cylinder_tree():
    """The reference's CylinderDivider (float build) on the configuration of
    examples/ParametricDivider/log_cylinder.4: root grid 1x1x2, levels 0..4,
    axis through (0.5, 0.5), r = 0.4, Hilbert."""
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "t.bin"
        subprocess.run([str(DRV / "refvc_f"), "tree", "1", "1", "2", "0",
                        "cylinder:0.5,0.5,0.4", "0", "4", "H", "2", str(out)], check=True)
        d, _ = read_blocks(out.read_bytes())
    np.savez_compressed(HERE / "tree_cylinder_1x1x2.npz", nb=d["nb"], pedigrees=d["pedigrees"],
                        levels=d["levels"], ld=d["ld"], id=d["id"], sf=d["sf"])
    print("tree_cylinder_1x1x2", d["nb"], "blocks")


def vc_mesh():
    """Pedigree list of the VC fixture mesh: 2x2x2 roots (periodic in x),
    sphere-surface refinement to level 2, 2:1 balanced -- every face kind."""
    import bcmtools_gb300 as bg
    rg = bg.RootGrid(2, 2, 2, periodic=(True, False, False), root_length=0.5)
    tree = bg.Octree.build(rg, bg.Divider.sphere_surface((0.5, 0.5, 0.5), 0.32, 2), "Z")
    return rg, tree


def gen_vc():
    rg, tree = vc_mesh()
    peds = tree.pedigrees
    for tname, drv in (("f32", "refvc_f"), ("f64", "refvc_d")):
        for n, vc in ((4, 1), (4, 2)):
            seed = 1000 + n * 10 + vc
            with tempfile.TemporaryDirectory() as td:
                pf = Path(td) / "p.bin"
                peds.astype(np.uint64).tofile(pf)
                out = Path(td) / "o.bin"
                subprocess.run([str(DRV / drv), "vc", "2", "2", "2", "1", str(pf), str(n),
                                str(vc), str(seed), str(out)], check=True)
                buf = out.read_bytes()
            d, off = read_blocks(buf)
            dt = np.float32 if tname == "f32" else np.float64
            n0 = n + 2 * vc
            cnt = d["nb"] * n0 ** 3
            before = np.frombuffer(buf, dt, cnt, off).reshape(d["nb"], n0, n0, n0)
            after = np.frombuffer(buf, dt, cnt, off + before.nbytes).reshape(before.shape)
            regen = splitmix_uniform(seed, cnt).astype(dt).reshape(before.shape)
            assert np.array_equal(regen, before), "seeded fill mismatch"
            np.savez_compressed(HERE / f"vc_{tname}_n{n}_vc{vc}.npz", n=n, vc=vc, seed=seed,
                                pedigrees=peds, ld=d["ld"], id=d["id"], sf=d["sf"],
                                after=after)
            print(f"vc_{tname}_n{n}_vc{vc}", d["nb"], "blocks")


def ghost_digest(field: np.ndarray, n: int, vc: int) -> str:
    """SHA-256 of the interior and face-ghost cells (edges and corners are
    never written by the reference) of a padded field, little-endian."""
    import hashlib
import os
    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import face_mask
    sel = np.ascontiguousarray(field[:, face_mask(n, vc)])
    return hashlib.sha256(sel.astype(sel.dtype.newbyteorder("<")).tobytes()).hexdigest()


def gen_vc_digests():
    """VC updates at the larger block edges and ghost widths the GPU tests use
    (8 cells with vc = 3, 16 cells with vc = 2): a SHA-256 of the result and
    a sample of whole blocks, since the full fields would be megabytes."""
    rg, tree = vc_mesh()
    peds = tree.pedigrees
    for tname, drv in (("f32", "refvc_f"), ("f64", "refvc_d")):
        for n, vc in ((8, 3), (16, 2)):
            seed = 1000 + n * 10 + vc
            with tempfile.TemporaryDirectory() as td:
                pf = Path(td) / "p.bin"
                peds.astype(np.uint64).tofile(pf)
                out = Path(td) / "o.bin"
                subprocess.run([str(DRV / drv), "vc", "2", "2", "2", "1", str(pf), str(n),
                                str(vc), str(seed), str(out)], check=True)
                buf = out.read_bytes()
            d, off = read_blocks(buf)
            dt = np.float32 if tname == "f32" else np.float64
            n0 = n + 2 * vc
            cnt = d["nb"] * n0 ** 3
            before = np.frombuffer(buf, dt, cnt, off).reshape(d["nb"], n0, n0, n0)
            after = np.frombuffer(buf, dt, cnt, off + before.nbytes).reshape(before.shape)
            regen = splitmix_uniform(seed, cnt).astype(dt).reshape(before.shape)
            assert np.array_equal(regen, before), "seeded fill mismatch"
            sample = np.arange(0, d["nb"], 96)
            np.savez_compressed(HERE / f"vcd_{tname}_n{n}_vc{vc}.npz", n=n, vc=vc, seed=seed,
                                pedigrees=peds, ld=d["ld"], id=d["id"], sf=d["sf"],
                                digest=ghost_digest(after, n, vc), sample_blocks=sample,
                                sample_after=after[sample])
            print(f"vcd_{tname}_n{n}_vc{vc}", d["nb"], "blocks")


def gen_sor1():
    conf = REF / "examples" / "sor1" / "test.conf"
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "s.bin"
        r = subprocess.run([str(DRV / "refsor1"), str(conf), str(out)], check=True,
                           capture_output=True, text=True)
        buf = out.read_bytes()
    err = [l for l in r.stdout.splitlines() if "errorMax" in l][-1]
    d, off = read_blocks(buf, with_bc=True)
    nb, n, vc = (int(x) for x in d["hdr"])
    n0 = n + 2 * vc
    field = np.frombuffer(buf, np.float64, nb * n0 ** 3, off).reshape(nb, n0, n0, n0)
    np.savez_compressed(HERE / "sor1.npz", n=n, vc=vc, omega=1.2, n_outer=400, n_inner=1,
                        b0=0.0, b1=1.0, error_max_line=err, pedigrees=d["pedigrees"],
                        cell_sizes=d["sizes"], origins=d["origins"], bc_type=d["bc_type"],
                        bc_id=d["bc_id"], ld=d["ld"], id=d["id"], sf=d["sf"], field=field)
    print("sor1", nb, "blocks;", err)


def gen_sor2():
    conf = REF / "examples" / "sor2" / "test.conf"
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "s.bin"
        subprocess.run([str(DRV / "refsor2"), str(conf), str(out)], check=True,
                       capture_output=True, text=True)
        buf = out.read_bytes()
    d, off = read_blocks(buf, with_bc=True)
    nb, n, vc = (int(x) for x in d["hdr"])
    n0 = n + 2 * vc
    field = np.frombuffer(buf, np.float64, nb * n0 ** 3, off).reshape(nb, n0, n0, n0)
    off += field.nbytes
    fac = np.frombuffer(buf, np.float64, nb * 3 * n, off).reshape(nb, 3, n)
    assert off + fac.nbytes == len(buf)
    sample = np.arange(0, nb, 29)
    np.savez_compressed(HERE / "sor2.npz", n=n, vc=vc, omega=1.4, n_outer=400, n_inner=1,
                        pedigrees=d["pedigrees"], cell_sizes=d["sizes"], origins=d["origins"],
                        bc_type=d["bc_type"], bc_id=d["bc_id"], ld=d["ld"], id=d["id"],
                        sf=d["sf"], source_factors=fac,
                        field_sha256=ghost_digest(field, n, vc), sample_blocks=sample,
                        sample_field=field[sample])
    print("sor2", nb, "blocks")


if __name__ == "__main__":
    gen_trees()
    gen_sphere_tree()
    gen_cylinder_tree()
    gen_vc()
    gen_vc_digests()
    gen_sor1()
    gen_sor2()
