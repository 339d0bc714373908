"""Builds libbcmg.so, the CUDA library behind include/bcmg.h, in-tree.

Each translation unit is compiled in parallel with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) and linked into
``bcmtools_gb300/_lib/libbcmg.so``.  No cmake, no torch extension machinery:
the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libbcmg.so"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-I", str(ROOT / "include"), "-I", str(CSRC)]
SOURCES = ["capi.cu", "vc.cu", "stencil.cu", "octree.cpp", "sor_f32.cu", "sor_f64.cu",
           "sor_f32_n8.cu", "sor_f32_n16.cu", "sor_f32_n32.cu", "sor_f64_n8.cu", "sor_f64_n16.cu",
           "sor_f64_n32.cu", "jacobi_f32.cu", "jacobi_f64.cu", "divcheck.cu", "krylov.cu",
           "mesh_dev.cu", "exchange.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbcmg.so")


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [_nvcc(), *GENCODE, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        # host code: no multiply-add contraction (the dividers' float and
        # double tests must decide as the device's do)
        cmd = [_nvcc(), *NVCC_FLAGS, "-Xcompiler", "-ffp-contract=off", *extra, "-x", "c++",
               "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.iterdir()) + [ROOT / "include" / "bcmg.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link libbcmg.so if any source is newer than the library."""
    if not force and not _stale():
        return LIB
    extra = extra or []
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for s in SOURCES:
            src = CSRC / s
            obj = objdir / (src.stem + ".o")
            jobs.append(ex.submit(_compile, src, obj, extra))
        for j in jobs:
            j.result()
    objs = [str(objdir / (Path(s).stem + ".o")) for s in SOURCES]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *GENCODE, "-shared", "-o", str(tmp), *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
