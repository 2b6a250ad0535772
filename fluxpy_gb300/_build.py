"""Build recipes for the native parts of fluxpy_gb300.

* ``libfluxgb.so``: every ``csrc/*.cu`` compiled with nvcc for sm_103a only
  (``-gencode arch=compute_103a,code=sm_103a``), one object per translation
  unit compiled in parallel, linked into one C-ABI shared library in the
  package directory (in-tree, loaded with ctypes).
* The checker libraries under ``oracle/`` are test infrastructure and are
  built by ``oracle/build.py``, never from this module.

Objects are cached in ``fluxpy_gb300/_build`` and rebuilt when a source or a
header is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
INCLUDE_DIR = REPO_DIR / "include"
LIB_PATH = PKG_DIR / "libfluxgb.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr", "-Xptxas", "-v",
]
# Translation units whose results must be bit-identical to plain IEEE C
# arithmetic (no FMA contraction): the conduction steps (plain and per-facet
# thermal inertia), the facet geometry, the ray/triangle predicates and the
# exact triangle view factor (whose parallel-edge terms cancel strongly, so
# contraction choices would make its two kernels differ in the last bits).
NO_FMAD = {"conduction.cu", "adjoint.cu", "geometry.cu", "raycast.cu", "formfactor.cu",
           "viewfactor.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfluxgb.so")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE_DIR.glob("*.h"))


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile_one(src: Path, verbose: bool) -> tuple[Path, str]:
    obj = BUILD_DIR / (src.stem + ".o")
    if not _newer(obj, [src, *_headers()]):
        return obj, ""
    flags = list(COMMON_FLAGS)
    if src.name in NO_FMAD:
        flags += ["-fmad=false"]
    cmd = [_nvcc(), *ARCH_FLAGS, *flags, "-I", str(INCLUDE_DIR), "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build_lib(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile csrc/*.cu for sm_103a and link libfluxgb.so (in-tree)."""
    BUILD_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile_one(s, verbose), sources))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log:
                (BUILD_DIR / (o.stem + ".ptxas.txt")).write_text(log)
    if _newer(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH_FLAGS, "-shared", "-Xcompiler", "-fPIC", *map(str, objs),
               "-o", str(tmp), "-lcuda"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build_lib(verbose="-v" in sys.argv)
    print(LIB_PATH)
