"""ctypes binding of include/bcmg.h (the C ABI of libbcmg.so).

Loading fails loudly when the library has not been built: there is no CPU
fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libbcmg.so"

SUCCESS, FAILURE, USAGE, MEMORY = 0, 1, 16, 17
NO_DEVICE, CUDA_ERROR, DIVERGED, NOT_CONVERGED, BREAKDOWN, SCRATCH_LIMIT = 40, 41, 42, 43, 44, 45
F32, F64 = 0, 1
KERNEL_KINDS = ("vc_gather", "sor_rb", "jacobi", "residual", "dot", "blas1", "fill", "other")
STATUS_NAMES = {0: "SUCCESS", 1: "FAILURE", 16: "USAGE", 17: "MEMORY", 20: "READ_DATA",
                21: "WRITE_DATA", 40: "NO_DEVICE", 41: "CUDA_ERROR", 42: "DIVERGED",
                43: "NOT_CONVERGED", 44: "BREAKDOWN", 45: "SCRATCH_LIMIT"}


class BcmgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"bcmg error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


class XchEntryC(C.Structure):
    _fields_ = [("block", C.c_int), ("face", C.c_int), ("subface", C.c_int), ("kind", C.c_int)]


class RootGridC(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("periodic_mask", C.c_int),
                ("origin", C.c_double * 3), ("root_length", C.c_double)]


class DividerC(C.Structure):
    _fields_ = [("kind", C.c_int), ("min_level", C.c_int), ("max_level", C.c_int),
                ("direction_mask", C.c_int), ("center", C.c_double * 3), ("radius", C.c_double),
                ("points", C.POINTER(C.c_double)), ("npoints", C.c_int), ("balance", C.c_int),
                ("margin_ratio", C.c_double)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("residual", C.c_double), ("status", C.c_int),
                ("refinements", C.c_int), ("true_residual", C.c_double),
                ("fp64_iterations", C.c_int)]


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
_U64P = C.POINTER(C.c_uint64)

# name -> (restype, argtypes)
_SIGS = {
    "bcmg_octree_build": (_I, [C.POINTER(_P), C.POINTER(RootGridC), C.POINTER(DividerC), _I,
                               C.c_uint64]),
    "bcmg_octree_from_pedigrees": (_I, [C.POINTER(_P), C.POINTER(RootGridC), _U64P, _I]),
    "bcmg_octree_num_leaves": (_I, [_P, _IP]),
    "bcmg_octree_leaves": (_I, [_P, _U64P, _IP, _DP, _DP]),
    "bcmg_octree_neighbors": (_I, [_P, _IP, _IP, _IP, _IP]),
    "bcmg_octree_destroy": (None, [_P]),
    "bcmg_ctx_create": (_I, [C.POINTER(_P), _I]),
    "bcmg_ctx_destroy": (None, [_P]),
    "bcmg_last_error": (C.c_char_p, [_P]),
    "bcmg_sync": (_I, [_P, _P]),
    "bcmg_set_memory_budget": (_I, [_P, C.c_size_t]),
    "bcmg_memory_in_use": (_I, [_P, C.POINTER(C.c_size_t)]),
    "bcmg_register_blocks": (_I, [_P, _I, _I, _I, _I, _IP, _IP, _IP]),
    "bcmg_mesh_build": (_I, [_P, C.POINTER(RootGridC), C.POINTER(DividerC), _I, _I, _I]),
    "bcmg_mesh_build_batch": (_I, [_P, _I, C.POINTER(RootGridC), C.POINTER(DividerC), _I, _I,
                                   _I, _IP]),
    "bcmg_mesh_register_pedigrees": (_I, [_P, C.POINTER(RootGridC), _U64P, _I, _I, _I, _I, _I]),
    "bcmg_mesh_pedigrees": (_I, [_P, _U64P]),
    "bcmg_num_blocks": (_I, [_P, _IP]),
    "bcmg_xch_bytes": (_I, [_P, _I, C.POINTER(XchEntryC), _I, C.POINTER(C.c_size_t)]),
    "bcmg_xch_pack": (_I, [_P, _I, C.POINTER(XchEntryC), _I, _P, _P]),
    "bcmg_xch_unpack": (_I, [_P, _I, C.POINTER(XchEntryC), _I, _P, _P]),
    "bcmg_mesh_neighbors": (_I, [_P, _IP, _IP, _IP, _IP]),
    "bcmg_set_boundary": (_I, [_P, _IP, _DP, _I]),
    "bcmg_set_segments": (_I, [_P, _I, _IP]),
    "bcmg_field_create": (_I, [_P, _I, _I, _IP]),
    "bcmg_field_create_host": (_I, [_P, _I, _I, _IP]),
    "bcmg_field_destroy": (_I, [_P, _I]),
    "bcmg_field_layout": (_I, [_P, _I, C.POINTER(_P), C.POINTER(C.c_int64),
                               C.POINTER(C.c_int64)]),
    "bcmg_field_upload": (_I, [_P, _I, _P, _P]),
    "bcmg_field_download": (_I, [_P, _I, _P, _P]),
    "bcmg_field_fill": (_I, [_P, _I, _D, _P]),
    "bcmg_field_copy": (_I, [_P, _I, _I, _P]),
    "bcmg_field_swap": (_I, [_P, _I, _I]),
    "bcmg_prepare_vc": (_I, [_P, _I, _I, _I]),
    "bcmg_vc_begin": (_I, [_P, _I, _I, _I, _P]),
    "bcmg_vc_end": (_I, [_P, _I]),
    "bcmg_bc_apply": (_I, [_P, _I, _P]),
    "bcmg_impose_bc": (_I, [_P, _I, _P]),
    "bcmg_sor_run": (_I, [_P, _I, _I, _DP, _D, _I, _I, _I, _P]),
    "bcmg_set_fusion": (_I, [_P, _I]),
    "bcmg_set_ghost_form": (_I, [_P, _I]),
    "bcmg_set_jacobi_shape": (_I, [_P, _I]),
    "bcmg_field_fill_random": (_I, [_P, _I, _I, _I, C.c_uint64, _D, _D, _P]),
    "bcmg_set_sor_variant": (_I, [_P, _I]),
    "bcmg_autotune_sor": (_I, [_P, _I, _I, _DP, _D, _I, _I, _IP, _DP]),
    "bcmg_autotune_jacobi": (_I, [_P, _I, _I, _I, _D, _I, _IP, _DP]),
    "bcmg_op_create_const": (_I, [_P, _DP, _IP]),
    "bcmg_op_create_fields": (_I, [_P, _IP, _IP]),
    "bcmg_op_destroy": (_I, [_P, _I]),
    "bcmg_op_fold_boundary": (_I, [_P, _I, _I, _P]),
    "bcmg_jacobi_sweep": (_I, [_P, _I, _I, _I, _I, _D, _P]),
    "bcmg_jacobi_run": (_I, [_P, _I, _I, _I, _D, _I, _I, _P]),
    "bcmg_calc_ax": (_I, [_P, _I, _I, _I, _P]),
    "bcmg_calc_r": (_I, [_P, _I, _I, _I, _I, _P]),
    "bcmg_calc_r2": (_I, [_P, _I, _I, _I, _DP, _P]),
    "bcmg_dot": (_I, [_P, _I, _I, _DP, _P]),
    "bcmg_dot_noalloc": (_I, [_I, _P, _P, _I, _I, _I, _I, _I, C.c_int64, _P, _P]),
    "bcmg_axpy": (_I, [_P, _I, _I, _D, _P]),
    "bcmg_xpay": (_I, [_P, _I, _I, _D, _P]),
    "bcmg_axpyz": (_I, [_P, _I, _I, _I, _D, _P]),
    "bcmg_axpbypz": (_I, [_P, _I, _I, _I, _D, _D, _P]),
    "bcmg_jacobi_solve": (_I, [_P, _I, _I, _I, _D, _I, _D, C.POINTER(SolveInfo), _P]),
    "bcmg_bicgstab": (_I, [_P, _I, _I, _I, _D, _I, _I, _D, C.POINTER(SolveInfo), _P]),
    "bcmg_bicgstab_mixed": (_I, [_P, _I, _I, _I, _D, _I, _I, _D, _I, _D, C.POINTER(SolveInfo),
                                 _P]),
    "bcmg_profile_begin": (_I, [_P]),
    "bcmg_profile_end": (_I, [_P, _DP, C.POINTER(C.c_int64)]),
    "bcmg_launch_count": (_I, [_P, C.POINTER(C.c_int64)]),
    "bcmg_check_division": (_I, [C.c_uint64, C.c_int64, C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64)]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load() -> C.CDLL:
    """Load libbcmg.so (once) and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
            f"g.build()\"` (no CPU fallback exists)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array."""
    return a.ctypes.data_as(C.POINTER(ctype))
