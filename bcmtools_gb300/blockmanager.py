"""Host-side mirror of the reference's BlockManager / Scalar3D<T> / VCUpdater
API (include/BlockManager.h, include/Scalar3D.h, include/VCUpdater.h) over the
C ABI of libbcmg.so.  Names and argument meaning follow the reference; errors
raise BcmgError instead of exiting.  Every data-parallel step runs in the
library's CUDA kernels; nothing here computes on field data.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import BcmgError
from .mesh import DeviceMesh, Divider, Octree, RootGrid

X_M, X_P, Y_M, Y_P, Z_M, Z_P = range(6)
BC_INNER, BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = range(4)
DIRICHLET_SOR, DIRICHLET_BCX = 0, 1
_DT = {"f32": (capi.F32, np.float32), "f64": (capi.F64, np.float64),
       np.float32: (capi.F32, np.float32), np.float64: (capi.F64, np.float64)}


class VCUpdateMethod:
    """VCUpdateMethod::Type (BlockManager.h:40-47)."""
    AtOnce = 0
    SeparateXYZ = 1
    SeparateXYZ_SeparateLevelDiff = 2


class Scalar3D:
    """A Scalar3D<T> data class registered on every block (one device arena).

    Host arrays use the reference brick layout: shape (nb, nz+2vc, ny+2vc,
    nx+2vc), x fastest; cell (i,j,k) of block b is a[b, k+vc, j+vc, i+vc]."""

    def __init__(self, bm: "BlockManager", handle: int, dtype, vc: int):
        self.bm, self.id, self.vc = bm, handle, vc
        self.dcode, self.dtype = _DT[dtype]
        n = bm.size
        self.shape = (bm.nb, n[2] + 2 * vc, n[1] + 2 * vc, n[0] + 2 * vc)

    def layout(self):
        p, s, e = C.c_void_p(), C.c_int64(), C.c_int64()
        self.bm._ck(self.bm.lib.bcmg_field_layout(self.bm.ctx, self.id, C.byref(p), C.byref(s),
                                                  C.byref(e)))
        return p.value, s.value, e.value

    def upload(self, a: np.ndarray, stream=None):
        a = np.ascontiguousarray(a, dtype=self.dtype).reshape(self.shape)
        self.bm._ck(self.bm.lib.bcmg_field_upload(self.bm.ctx, self.id, a.ctypes.data, stream))
        self.bm.sync(stream)

    def download(self, stream=None) -> np.ndarray:
        a = np.empty(self.shape, self.dtype)
        self.bm._ck(self.bm.lib.bcmg_field_download(self.bm.ctx, self.id, a.ctypes.data, stream))
        return a

    def fill(self, v: float, stream=None):
        self.bm._ck(self.bm.lib.bcmg_field_fill(self.bm.ctx, self.id, float(v), stream))

    def fill_random(self, seed: int, lo=-1.0, hi=1.0, first_block=0, nblocks=None, stream=None):
        """Seeded uniform [lo, hi) interior values on a block range (ghosts kept)."""
        nb = self.bm.nb - first_block if nblocks is None else nblocks
        self.bm._ck(self.bm.lib.bcmg_field_fill_random(self.bm.ctx, self.id, int(first_block),
                                                       int(nb), int(seed), float(lo), float(hi),
                                                       stream))

    def interior(self, a: np.ndarray) -> np.ndarray:
        v = self.vc
        return a[:, v:-v, v:-v, v:-v]

    def dump(self, step: int, label: str, directory: str = "BIN", rank: int = 0):
        """LocalScalar3D::Dump (SolverTest/LocalScalar3D.cpp:85-134): ghosts
        imposed, then one file per block (bcmtools_gb300.dump)."""
        from .dump import write_blocks
        self.bm.imposeBoundaryCondition(self)
        write_blocks(self.download(), self.vc, directory, label, step, rank)

    def load(self, step: int, label: str, directory: str = "BIN", rank: int = 0):
        """LocalScalar3D::Load (SolverTest/LocalScalar3D.cpp:136-222): blocks of
        the same size, or of half the cells per axis (injected), then the
        boundary conditions imposed."""
        from .dump import read_blocks
        a = read_blocks(self.shape, self.vc, directory, label, step, rank, self.dtype,
                        out=self.download())
        self.upload(a)
        self.bm.imposeBoundaryCondition(self)


class BlockManager:
    """BlockManager (include/BlockManager.h:56-875) for one GPU, one rank."""

    def __init__(self, device: int = 0):
        self.lib = capi.load()
        self.ctx = C.c_void_p()
        self.device = device
        rc = self.lib.bcmg_ctx_create(C.byref(self.ctx), device)
        if rc != 0:
            raise BcmgError(rc, "bcmg_ctx_create: no usable CUDA device")
        self.nb = 0
        self.size = None

    # -- errors / sync -----------------------------------------------------
    def _ck(self, rc):
        if rc != 0:
            raise BcmgError(rc, self.lib.bcmg_last_error(self.ctx).decode())
        return rc

    def sync(self, stream=None):
        self._ck(self.lib.bcmg_sync(self.ctx, stream))

    def launch_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.bcmg_launch_count(self.ctx, C.byref(n)))
        return n.value

    def profile_begin(self):
        """Start per-launch CUDA-event timing (bcmg_profile_begin)."""
        self._ck(self.lib.bcmg_profile_begin(self.ctx))

    def profile_end(self) -> dict:
        """{kernel kind: (total ms, launches)} since profile_begin."""
        ms = (C.c_double * 8)()
        cnt = (C.c_int64 * 8)()
        self._ck(self.lib.bcmg_profile_end(self.ctx, ms, cnt))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(capi.KERNEL_KINDS)}

    def set_memory_budget(self, nbytes: int):
        self._ck(self.lib.bcmg_set_memory_budget(self.ctx, int(nbytes)))

    def memory_in_use(self) -> int:
        n = C.c_size_t()
        self._ck(self.lib.bcmg_memory_in_use(self.ctx, C.byref(n)))
        return n.value

    # -- registration ------------------------------------------------------
    def register_blocks(self, ld, nid, sf, size):
        """registerBlock x nb + endRegisterBlock (BlockManager.cpp:28-59)."""
        ld = np.ascontiguousarray(ld, np.int32)
        nid = np.ascontiguousarray(nid, np.int32)
        sf = np.ascontiguousarray(sf, np.int32)
        nb = ld.shape[0]
        n = (size, size, size) if np.isscalar(size) else tuple(size)
        self._ck(self.lib.bcmg_register_blocks(self.ctx, nb, n[0], n[1], n[2],
                                               capi.ptr(ld, C.c_int), capi.ptr(nid, C.c_int),
                                               capi.ptr(sf, C.c_int)))
        self.nb, self.size = nb, n

    def register_octree(self, tree: Octree, size):
        ld, nid, sf, outer = tree.neighbors()
        self.register_blocks(ld, nid, sf, size)
        self.tree, self.outer = tree, outer
        return outer

    # -- device-side mesh set-up --------------------------------------------
    def _adopt_device_mesh(self, rg, size, first=None):
        """The registered mesh's tables, read back as DeviceMesh objects (one
        per mesh of a batch, ids local to each)."""
        nb = self._num_registered()
        peds = np.zeros(nb, np.uint64)
        ld = np.zeros((nb, 6), np.int32)
        nid = np.zeros((nb, 6, 4), np.int32)
        sf = np.zeros((nb, 6), np.int32)
        outer = np.zeros((nb, 6), np.int32)
        self._ck(self.lib.bcmg_mesh_pedigrees(self.ctx, capi.ptr(peds, C.c_uint64)))
        self._ck(self.lib.bcmg_mesh_neighbors(self.ctx, capi.ptr(ld, C.c_int),
                                              capi.ptr(nid, C.c_int), capi.ptr(sf, C.c_int),
                                              capi.ptr(outer, C.c_int)))
        n = (size, size, size) if np.isscalar(size) else tuple(size)
        self.nb, self.size, self.outer = nb, n, outer
        if first is None:
            self.tree = DeviceMesh(rg, peds, ld, nid, sf, outer)
            return self.tree
        meshes = []
        bounds = list(first) + [nb]
        for k, r in enumerate(rg):
            a, b = bounds[k], bounds[k + 1]
            loc = np.where(nid[a:b] >= 0, nid[a:b] - a, nid[a:b])
            meshes.append(DeviceMesh(r, peds[a:b], ld[a:b], loc, sf[a:b], outer[a:b]))
        self.tree = None
        return meshes

    def _num_registered(self) -> int:
        n = C.c_int(0)
        self._ck(self.lib.bcmg_num_blocks(self.ctx, C.byref(n)))
        return n.value

    def build_mesh(self, rg: RootGrid, div: Divider, size) -> DeviceMesh:
        """The octree of `div` over `rg` made on the GPU (2:1 balanced when
        div.balance, leaves in Z order) and registered: the blocks, order and
        neighbour table Octree.build(rg, div, "Z") gives (bcmg_mesh_build)."""
        n = (size, size, size) if np.isscalar(size) else tuple(size)
        rgc, dc = rg.to_c(), div.to_c()
        self._ck(self.lib.bcmg_mesh_build(self.ctx, C.byref(rgc), C.byref(dc), n[0], n[1], n[2]))
        return self._adopt_device_mesh(rg, size)

    def build_mesh_batch(self, specs, size):
        """Meshes [(rg, div), ...] made on the GPU and registered as one block
        set, mesh k from block first[k] on (bcmg_mesh_build_batch).  Returns
        (first, [DeviceMesh per mesh])."""
        n = (size, size, size) if np.isscalar(size) else tuple(size)
        k = len(specs)
        rgs = (capi.RootGridC * k)(*[rg.to_c() for rg, _ in specs])
        divs = (capi.DividerC * k)(*[d.to_c() for _, d in specs])
        first = np.zeros(k, np.int32)
        self._ck(self.lib.bcmg_mesh_build_batch(self.ctx, k, rgs, divs, n[0], n[1], n[2],
                                                capi.ptr(first, C.c_int)))
        meshes = self._adopt_device_mesh([rg for rg, _ in specs], size, first)
        return [int(f) for f in first], meshes

    def register_pedigrees(self, rg: RootGrid, peds, size, balance: bool = False) -> DeviceMesh:
        """Blocks = the listed leaves in list order, neighbours found on the
        GPU (bcmg_mesh_register_pedigrees); with `balance`, the list refined
        2:1 on the GPU first, blocks then in Z order."""
        n = (size, size, size) if np.isscalar(size) else tuple(size)
        p = np.ascontiguousarray(np.asarray(peds, dtype=np.uint64))
        rgc = rg.to_c()
        self._ck(self.lib.bcmg_mesh_register_pedigrees(self.ctx, C.byref(rgc),
                                                       capi.ptr(p, C.c_uint64), len(p),
                                                       1 if balance else 0, n[0], n[1], n[2]))
        return self._adopt_device_mesh(rg, size)

    def set_boundary(self, bc_type, bc_value, form=DIRICHLET_SOR):
        t = np.ascontiguousarray(bc_type, np.int32).reshape(self.nb, 6)
        v = np.ascontiguousarray(bc_value, np.float64).reshape(self.nb, 6)
        self._ck(self.lib.bcmg_set_boundary(self.ctx, capi.ptr(t, C.c_int),
                                            capi.ptr(v, C.c_double), form))

    def getNumBlock(self) -> int:
        return self.nb

    def printBlockLayoutInfo(self, file=None):
        """BlockManager::printBlockLayoutInfo (BlockManager.cpp:118-288) for a
        mesh registered from an octree: blocks per level and faces by level
        difference, this process being the one rank."""
        import sys
        from .mesh import format_layout_info, layout_info
        if getattr(self, "tree", None) is None:
            raise BcmgError(capi.USAGE, "block levels are known for octree meshes only")
        ld, nid, _, _ = self.tree.neighbors()
        print(format_layout_info(layout_info(self.tree.levels, ld, nid)),
              file=file or sys.stdout)

    def getSize(self):
        return self.size

    # -- data classes ------------------------------------------------------
    def setDataClass(self, dtype="f32", vc=1) -> Scalar3D:
        """setDataClass<Scalar3D<T>, Scalar3DUpdater<T>>(vc) (BlockManager.h:226-247)."""
        h = C.c_int()
        self._ck(self.lib.bcmg_field_create(self.ctx, _DT[dtype][0], vc, C.byref(h)))
        return Scalar3D(self, h.value, dtype, vc)

    def destroy(self, f: Scalar3D):
        self._ck(self.lib.bcmg_field_destroy(self.ctx, f.id))

    def prepareForVCUpdate(self, f: Scalar3D, tag: int = 100,
                           method: int = VCUpdateMethod.AtOnce):
        self._ck(self.lib.bcmg_prepare_vc(self.ctx, f.id, tag, method))

    # -- VC update (BlockManager.h:311-726) ---------------------------------
    def beginUpdateVC(self, f, axis_mask=7, ld_mask=7, stream=None):
        self._ck(self.lib.bcmg_vc_begin(self.ctx, f.id, axis_mask, ld_mask, stream))

    def endUpdateVC(self, f):
        self._ck(self.lib.bcmg_vc_end(self.ctx, f.id))

    def updateVC(self, f, axis_mask=7, ld_mask=7):
        self.beginUpdateVC(f, axis_mask, ld_mask)
        self.endUpdateVC(f)

    def updateVC_X(self, f): self.updateVC(f, 1)
    def updateVC_Y(self, f): self.updateVC(f, 2)
    def updateVC_Z(self, f): self.updateVC(f, 4)
    def updateVC_Flat(self, f, xyz): self.updateVC(f, 1 << xyz, 2)
    def updateVC_F2C(self, f, xyz): self.updateVC(f, 1 << xyz, 4)
    def updateVC_C2F(self, f, xyz): self.updateVC(f, 1 << xyz, 1)

    # Per-axis and per-level-difference begin/end pairs (BlockManager.h:
    # 321-670): xyz 0/1/2 is the axis; Flat = same level, F2C = from finer
    # neighbours (level difference +1), C2F = from coarser ones (-1).  Several
    # begins may precede their ends (sor2's separateVCUpdate order); every
    # begin is stream-ordered and an end waits for the field's latest begin.
    def beginUpdateVC_X(self, f, stream=None): self.beginUpdateVC(f, 1, 7, stream)
    def beginUpdateVC_Y(self, f, stream=None): self.beginUpdateVC(f, 2, 7, stream)
    def beginUpdateVC_Z(self, f, stream=None): self.beginUpdateVC(f, 4, 7, stream)
    def endUpdateVC_X(self, f): self.endUpdateVC(f)
    def endUpdateVC_Y(self, f): self.endUpdateVC(f)
    def endUpdateVC_Z(self, f): self.endUpdateVC(f)

    def beginUpdateVC_Flat(self, f, xyz, stream=None): self.beginUpdateVC(f, 1 << xyz, 2, stream)
    def beginUpdateVC_F2C(self, f, xyz, stream=None): self.beginUpdateVC(f, 1 << xyz, 4, stream)
    def beginUpdateVC_C2F(self, f, xyz, stream=None): self.beginUpdateVC(f, 1 << xyz, 1, stream)
    def endUpdateVC_Flat(self, f, xyz): self.endUpdateVC(f)
    def endUpdateVC_F2C(self, f, xyz): self.endUpdateVC(f)
    def endUpdateVC_C2F(self, f, xyz): self.endUpdateVC(f)

    def updateVC_X_Flat(self, f): self.updateVC_Flat(f, 0)
    def updateVC_Y_Flat(self, f): self.updateVC_Flat(f, 1)
    def updateVC_Z_Flat(self, f): self.updateVC_Flat(f, 2)
    def updateVC_X_F2C(self, f): self.updateVC_F2C(f, 0)
    def updateVC_Y_F2C(self, f): self.updateVC_F2C(f, 1)
    def updateVC_Z_F2C(self, f): self.updateVC_F2C(f, 2)
    def updateVC_X_C2F(self, f): self.updateVC_C2F(f, 0)
    def updateVC_Y_C2F(self, f): self.updateVC_C2F(f, 1)
    def updateVC_Z_C2F(self, f): self.updateVC_C2F(f, 2)

    def setBoundaryCondition(self, f, stream=None):
        self._ck(self.lib.bcmg_bc_apply(self.ctx, f.id, stream))

    def imposeBoundaryCondition(self, f, stream=None):
        self._ck(self.lib.bcmg_impose_bc(self.ctx, f.id, stream))

    # -- sweeps and solvers -------------------------------------------------
    def set_sor_variant(self, variant: int):
        """Force a fused-SOR kernel shape (0 = automatic); see bcmg_set_sor_variant."""
        self._ck(self.lib.bcmg_set_sor_variant(self.ctx, int(variant)))

    def autotune_sor(self, f, coef, omega, form=1, s=None, iters=20):
        """Time every fused-SOR kernel shape on a copy of f; keep the fastest."""
        cf = np.ascontiguousarray(coef, np.float64).reshape(self.nb, 4)
        best, us = C.c_int(), C.c_double()
        self._ck(self.lib.bcmg_autotune_sor(self.ctx, f.id, s.id if s is not None else -1,
                                            capi.ptr(cf, C.c_double), float(omega), form, iters,
                                            C.byref(best), C.byref(us)))
        return best.value, us.value

    def set_fusion(self, enable: bool):
        """Fused sweep + ghost update (default) or separate launches."""
        self._ck(self.lib.bcmg_set_fusion(self.ctx, 1 if enable else 0))

    def set_ghost_form(self, push=None):
        """Ghost form of the fused sweeps: True push, False pull, None automatic."""
        form = 2 if push is None else (1 if push else 0)
        self._ck(self.lib.bcmg_set_ghost_form(self.ctx, form))

    def set_jacobi_shape(self, shape: int):
        """Pull-form Jacobi kernel: 0 automatic, 1 one CTA per block, 2 pipelined."""
        self._ck(self.lib.bcmg_set_jacobi_shape(self.ctx, int(shape)))

    def sor_run(self, f, coef, omega, form=1, n_inner=1, n_outer=1, s=None, stream=None):
        cf = np.ascontiguousarray(coef, np.float64).reshape(self.nb, 4)
        self._ck(self.lib.bcmg_sor_run(self.ctx, f.id, s.id if s is not None else -1,
                                       capi.ptr(cf, C.c_double), float(omega), form, n_inner,
                                       n_outer, stream))

    def op_const(self, cc) -> int:
        cc = np.ascontiguousarray(cc, np.float64).reshape(self.nb, 7)
        h = C.c_int()
        self._ck(self.lib.bcmg_op_create_const(self.ctx, capi.ptr(cc, C.c_double), C.byref(h)))
        return h.value

    def op_fields(self, fields7) -> int:
        ids = np.array([f.id for f in fields7], np.int32)
        h = C.c_int()
        self._ck(self.lib.bcmg_op_create_fields(self.ctx, capi.ptr(ids, C.c_int), C.byref(h)))
        return h.value

    def fold_boundary(self, op, b, stream=None):
        """LocalScalar3D::ImposeBoundaryCondition(Ap..At, b) (SolverTest
        LocalScalar3D.h:260-285): folds the outer Dirichlet / Neumann faces
        of the boundary table into the coefficient fields of `op` and `b`."""
        self._ck(self.lib.bcmg_op_fold_boundary(self.ctx, op, b.id, stream))

    def jacobi_sweep(self, op, x1, x0, b, omega, stream=None):
        self._ck(self.lib.bcmg_jacobi_sweep(self.ctx, op, x1.id, x0.id, b.id, float(omega),
                                            stream))

    def autotune_jacobi(self, op, x, b, omega, iters=20):
        """Time the fused-Jacobi choices (1 push, 2 pull one CTA per block,
        3 pull pipelined) on a copy of x; keep the fastest."""
        best, us = C.c_int(), C.c_double()
        self._ck(self.lib.bcmg_autotune_jacobi(self.ctx, op, x.id, b.id, float(omega), int(iters),
                                               C.byref(best), C.byref(us)))
        return best.value, us.value

    def jacobi_run(self, op, x, b, omega, n_iter, use_graph=False, stream=None):
        """n_iter fused Jacobi sweeps with ghost update (bcmg_jacobi_run)."""
        self._ck(self.lib.bcmg_jacobi_run(self.ctx, op, x.id, b.id, float(omega), int(n_iter),
                                          1 if use_graph else 0, stream))

    def calc_ax(self, op, ax, x, stream=None):
        self._ck(self.lib.bcmg_calc_ax(self.ctx, op, ax.id, x.id, stream))

    def calc_r(self, op, r, x, b, stream=None):
        self._ck(self.lib.bcmg_calc_r(self.ctx, op, r.id, x.id, b.id, stream))

    def calc_r2(self, op, x, b, stream=None) -> float:
        v = C.c_double()
        self._ck(self.lib.bcmg_calc_r2(self.ctx, op, x.id, b.id, C.byref(v), stream))
        return v.value

    def dot(self, x, y, stream=None) -> float:
        v = C.c_double()
        self._ck(self.lib.bcmg_dot(self.ctx, x.id, y.id, C.byref(v), stream))
        return v.value

    def axpy(self, y, x, a, stream=None):
        self._ck(self.lib.bcmg_axpy(self.ctx, y.id, x.id, float(a), stream))

    def xpay(self, y, x, a, stream=None):
        self._ck(self.lib.bcmg_xpay(self.ctx, y.id, x.id, float(a), stream))

    def axpyz(self, z, x, y, a, stream=None):
        self._ck(self.lib.bcmg_axpyz(self.ctx, z.id, x.id, y.id, float(a), stream))

    def axpbypz(self, z, x, y, a, b, stream=None):
        self._ck(self.lib.bcmg_axpbypz(self.ctx, z.id, x.id, y.id, float(a), float(b), stream))

    def jacobi_solve(self, op, x, b, omega=1.0, max_iter=100, eps=1e-8, stream=None):
        info = capi.SolveInfo()
        rc = self.lib.bcmg_jacobi_solve(self.ctx, op, x.id, b.id, float(omega), max_iter,
                                        float(eps), C.byref(info), stream)
        if rc not in (0, capi.DIVERGED):
            self._ck(rc)
        return info

    def set_segments(self, seg_first):
        """Independent systems in one mesh (bcmg_set_segments): blocks
        [seg_first[s], seg_first[s+1]) form segment s; the BiCGSTAB solvers
        then return one SolveInfo per segment."""
        sf = np.ascontiguousarray(seg_first, np.int32)
        self._ck(self.lib.bcmg_set_segments(self.ctx, len(sf) - 1, capi.ptr(sf, C.c_int)))
        self.nseg = len(sf) - 1

    def _infos(self):
        n = getattr(self, "nseg", 1)
        return (capi.SolveInfo * n)()

    def bicgstab(self, op, x, b, omega=1.0, n_pre=2, max_iter=1000, eps=1e-8, stream=None):
        """ILS3D::BiCGSTAB; a SolveInfo, or a list of one per segment."""
        infos = self._infos()
        rc = self.lib.bcmg_bicgstab(self.ctx, op, x.id, b.id, float(omega), n_pre, max_iter,
                                    float(eps), infos, stream)
        if rc not in (0, capi.DIVERGED):
            self._ck(rc)
        return infos[0] if len(infos) == 1 else list(infos)

    def bicgstab_mixed(self, op, x, b, omega=1.0, n_pre=2, max_inner=200, eps_inner=1e-4,
                       max_outer=20, eps=1e-10, stream=None):
        """Mixed-precision BiCGSTAB; a SolveInfo, or a list of one per segment."""
        infos = self._infos()
        rc = self.lib.bcmg_bicgstab_mixed(self.ctx, op, x.id, b.id, float(omega), n_pre,
                                          max_inner, float(eps_inner), max_outer, float(eps),
                                          infos, stream)
        if rc not in (0, capi.DIVERGED):
            self._ck(rc)
        return infos[0] if len(infos) == 1 else list(infos)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.bcmg_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- coefficient helpers (what the reference's drivers compute per block) ----

def sor1_coef(cell_sizes: np.ndarray, omega: float) -> np.ndarray:
    """Per-block {c0, cx, cy, cz} of sor1 Solver::run (sor1/Solver.cpp:89-99)."""
    out = np.zeros((len(cell_sizes), 4))
    for b, (hx, hy, hz) in enumerate(np.asarray(cell_sizes, np.float64)):
        cx, cy, cz = 1.0 / (hx * hx), 1.0 / (hy * hy), 1.0 / (hz * hz)
        c = 2.0 * (cx + cy + cz)
        out[b] = (1.0 - omega, omega * cx / c, omega * cy / c, omega * cz / c)
    return out


def sor2_coef(cell_sizes: np.ndarray) -> np.ndarray:
    """Per-block {c, cx, cy, cz} of sor2 Solver::run (sor2/Solver.cpp:94-99)."""
    out = np.zeros((len(cell_sizes), 4))
    for b, (hx, hy, hz) in enumerate(np.asarray(cell_sizes, np.float64)):
        cx, cy, cz = 1.0 / (hx * hx), 1.0 / (hy * hy), 1.0 / (hz * hz)
        out[b] = (1.0 / (2.0 * (cx + cy + cz)), cx, cy, cz)
    return out


def laplace_coef(cell_sizes: np.ndarray) -> np.ndarray:
    """Per-block constant 7-point Laplacian {Ap, Aw, Ae, As, An, Ab, At}."""
    h = np.asarray(cell_sizes, np.float64)
    cx, cy, cz = 1.0 / h[:, 0] ** 2, 1.0 / h[:, 1] ** 2, 1.0 / h[:, 2] ** 2
    return np.stack([-2.0 * (cx + cy + cz), cx, cx, cy, cy, cz, cz], axis=1)
