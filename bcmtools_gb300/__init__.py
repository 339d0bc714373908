"""bcmtools_gb300 -- GB300 (sm_103a) implementation of the BCMTools ghost
(virtual cell) update over an octree of blocks and of the Jacobi, red-black
SOR and BiCGSTAB 7-point sweeps that drive it.

The product is libbcmg.so (CUDA + C++ host code behind the C ABI in
include/bcmg.h).  This package is its Python host mirror: the octree builder
(mesh), the BlockManager / Scalar3D API (blockmanager) and the ctypes binding
(capi).  There is no CPU fallback: every entry point that touches field data
runs the library's CUDA kernels, and importing fails if the library is absent.
"""
from .capi import BcmgError, load as _load_library
from .mesh import Divider, Octree, Partition, RootGrid, pedigree, unpack_pedigrees
from .blockmanager import (BC_DIRICHLET, BC_INNER, BC_NEUMANN, BC_PERIODIC, DIRICHLET_BCX,
                           DIRICHLET_SOR, BlockManager, Scalar3D, VCUpdateMethod, laplace_coef,
                           sor1_coef, sor2_coef)

_load_library()

__all__ = ["BcmgError", "Divider", "Octree", "Partition", "RootGrid", "pedigree",
           "unpack_pedigrees",
           "BlockManager", "Scalar3D", "VCUpdateMethod", "laplace_coef", "sor1_coef",
           "sor2_coef", "BC_INNER", "BC_DIRICHLET", "BC_NEUMANN", "BC_PERIODIC",
           "DIRICHLET_SOR", "DIRICHLET_BCX"]
