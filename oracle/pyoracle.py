"""ctypes binding of the CPU oracle (oracle/bcm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The GPU product never imports it.

Arrays use the packed brick layout (nb, nz+2vc, ny+2vc, nx+2vc), x fastest.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_c" / "libbcm_oracle.so"

_lib = None


def build() -> Path:
    """Compile the oracle library (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", str(HERE), str(LIB)], check=True)
    return LIB


class Mesh(C.Structure):
    _fields_ = [("nb", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("vc", C.c_int), ("bstride", C.c_long), ("nbr_id", C.POINTER(C.c_int)),
                ("nbr_ld", C.POINTER(C.c_int)), ("nbr_sf", C.POINTER(C.c_int))]


class Op(C.Structure):
    _fields_ = [("cc", C.POINTER(C.c_double)), ("A", C.c_void_p * 7)]


class Bc(C.Structure):
    _fields_ = [("bc_type", C.POINTER(C.c_int)), ("bc_value", C.POINTER(C.c_double)),
                ("form", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _lib.bcmo_calc_r2_f32.restype = C.c_double
        _lib.bcmo_calc_r2_f64.restype = C.c_double
        _lib.bcmo_dot_f32.restype = C.c_double
        _lib.bcmo_dot_f64.restype = C.c_double
        for t in ("f32", "f64"):
            for fn in ("jacobi_solve", "bicgstab"):
                getattr(_lib, f"bcmo_{fn}_{t}").restype = C.c_int
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _sfx(a):
    return "f32" if a.dtype == np.float32 else "f64"


def _ct(a):
    return C.c_float if a.dtype == np.float32 else C.c_double


class OracleMesh:
    """Block table + brick geometry, holding the arrays the C struct points to."""

    def __init__(self, ld, nid, sf, n, vc):
        self.ld = np.ascontiguousarray(ld, np.int32)
        self.id = np.ascontiguousarray(nid, np.int32)
        self.sf = np.ascontiguousarray(sf, np.int32)
        self.nb = self.ld.shape[0]
        self.n = (n, n, n) if np.isscalar(n) else tuple(n)
        self.vc = vc
        n0 = [x + 2 * vc for x in self.n]
        self.brick = n0[0] * n0[1] * n0[2]
        self.shape = (self.nb, n0[2], n0[1], n0[0])
        self.c = Mesh(self.nb, self.n[0], self.n[1], self.n[2], vc, self.brick,
                      _p(self.id, C.c_int), _p(self.ld, C.c_int), _p(self.sf, C.c_int))

    def zeros(self, dtype):
        return np.zeros(self.shape, dtype)

    # -- ghost update / boundary --------------------------------------------
    def vc_update(self, a, axis_mask=7, ld_mask=7):
        getattr(lib(), f"bcmo_vc_update_{_sfx(a)}")(C.byref(self.c), _p(a, _ct(a)), axis_mask,
                                                    ld_mask)

    def dirichlet(self, a, bc_type, bc_value, form=0):
        t = np.ascontiguousarray(bc_type, np.int32)
        v = np.ascontiguousarray(bc_value, np.float64)
        getattr(lib(), f"bcmo_dirichlet_{_sfx(a)}")(C.byref(self.c), _p(a, _ct(a)),
                                                    _p(t, C.c_int), _p(v, C.c_double), form)

    def fold(self, fields7, b, bc_type, bc_value):
        """Boundary folding of the coefficient bricks Ap..At and b, in place."""
        t = np.ascontiguousarray(bc_type, np.int32)
        v = np.ascontiguousarray(bc_value, np.float64)
        for a in list(fields7) + [b]:
            assert a.flags.c_contiguous and a.dtype == b.dtype
        arr = (C.c_void_p * 7)(*[a.ctypes.data for a in fields7])
        getattr(lib(), f"bcmo_fold_{_sfx(b)}")(C.byref(self.c), arr, _p(b, _ct(b)),
                                               _p(t, C.c_int), _p(v, C.c_double))

    def _bc(self, bc_type, bc_value, form):
        self._bct = np.ascontiguousarray(bc_type, np.int32)
        self._bcv = np.ascontiguousarray(bc_value, np.float64)
        return Bc(_p(self._bct, C.c_int), _p(self._bcv, C.c_double), form)

    def _op(self, cc=None, fields=None):
        o = Op()
        if cc is not None:
            self._cc = np.ascontiguousarray(cc, np.float64)
            o.cc = _p(self._cc, C.c_double)
        else:
            self._fields = [np.ascontiguousarray(f) for f in fields]
            for k in range(7):
                o.A[k] = self._fields[k].ctypes.data
        return o

    # -- sweeps --------------------------------------------------------------
    def sor_rb(self, f, coef, omega, form, s=None):
        cf = np.ascontiguousarray(coef, np.float64)
        sp = _p(s, _ct(f)) if s is not None else None
        getattr(lib(), f"bcmo_sor_rb_{_sfx(f)}")(C.byref(self.c), _p(f, _ct(f)), sp,
                                                 _p(cf, C.c_double), C.c_double(omega), form)

    def sor_run(self, f, coef, omega, form, n_inner, n_outer, bc_type, bc_value, bc_form=0,
                s=None):
        cf = np.ascontiguousarray(coef, np.float64)
        bc = self._bc(bc_type, bc_value, bc_form)
        sp = _p(s, _ct(f)) if s is not None else None
        getattr(lib(), f"bcmo_sor_run_{_sfx(f)}")(C.byref(self.c), C.byref(bc), _p(f, _ct(f)),
                                                  sp, _p(cf, C.c_double), C.c_double(omega),
                                                  form, n_inner, n_outer)

    def jacobi(self, x1, x0, b, omega, cc=None, fields=None):
        op = self._op(cc, fields)
        ct = _ct(x0)
        getattr(lib(), f"bcmo_jacobi_{_sfx(x0)}")(C.byref(self.c), C.byref(op), _p(x1, ct),
                                                  _p(x0, ct), _p(b, ct), ct(omega))

    def calc_ax(self, ax, x, cc=None, fields=None):
        op = self._op(cc, fields)
        getattr(lib(), f"bcmo_calc_ax_{_sfx(x)}")(C.byref(self.c), C.byref(op), _p(ax, _ct(x)),
                                                  _p(x, _ct(x)))

    def calc_r(self, r, x, b, cc=None, fields=None):
        op = self._op(cc, fields)
        ct = _ct(x)
        getattr(lib(), f"bcmo_calc_r_{_sfx(x)}")(C.byref(self.c), C.byref(op), _p(r, ct),
                                                 _p(x, ct), _p(b, ct))

    def calc_r2(self, x, b, cc=None, fields=None):
        op = self._op(cc, fields)
        ct = _ct(x)
        return getattr(lib(), f"bcmo_calc_r2_{_sfx(x)}")(C.byref(self.c), C.byref(op),
                                                         _p(x, ct), _p(b, ct))

    def dot(self, x, y):
        ct = _ct(x)
        return getattr(lib(), f"bcmo_dot_{_sfx(x)}")(C.byref(self.c), _p(x, ct), _p(y, ct))

    def blas1(self, kind, z, x, y=None, a=0.0, b=0.0):
        ct = _ct(z)
        L = lib()
        s = _sfx(z)
        if kind == "axpy":
            getattr(L, f"bcmo_axpy_{s}")(C.byref(self.c), _p(z, ct), _p(x, ct), ct(a))
        elif kind == "xpay":
            getattr(L, f"bcmo_xpay_{s}")(C.byref(self.c), _p(z, ct), _p(x, ct), ct(a))
        elif kind == "axpyz":
            getattr(L, f"bcmo_axpyz_{s}")(C.byref(self.c), _p(z, ct), _p(x, ct), _p(y, ct), ct(a))
        else:
            getattr(L, f"bcmo_axpbypz_{s}")(C.byref(self.c), _p(z, ct), _p(x, ct), _p(y, ct),
                                            ct(a), ct(b))

    # -- solvers ---------------------------------------------------------------
    def jacobi_solve(self, x, b, omega, max_iter, eps, bc_type, bc_value, bc_form=0, cc=None,
                     fields=None):
        op = self._op(cc, fields)
        bc = self._bc(bc_type, bc_value, bc_form)
        x0 = np.zeros_like(x)
        res = C.c_double()
        ct = _ct(x)
        it = getattr(lib(), f"bcmo_jacobi_solve_{_sfx(x)}")(
            C.byref(self.c), C.byref(op), C.byref(bc), _p(x, ct), _p(x0, ct), _p(b, ct),
            ct(omega), max_iter, C.c_double(eps), C.byref(res))
        return it, res.value

    def bicgstab(self, x, b, omega, n_pre, max_iter, eps, bc_type, bc_value, bc_form=0,
                 cc=None, fields=None):
        op = self._op(cc, fields)
        bc = self._bc(bc_type, bc_value, bc_form)
        work = np.zeros((9,) + x.shape, x.dtype)
        res = C.c_double()
        ct = _ct(x)
        it = getattr(lib(), f"bcmo_bicgstab_{_sfx(x)}")(
            C.byref(self.c), C.byref(op), C.byref(bc), _p(x, ct), _p(b, ct), _p(work, ct),
            ct(omega), n_pre, max_iter, C.c_double(eps), C.byref(res))
        return it, res.value


def num_threads() -> int:
    return lib().bcmo_num_threads()


def set_threads(n: int) -> None:
    """OpenMP threads of the oracle's loops (1: every sum in block order)."""
    lib().bcmo_set_threads(int(n))
