"""Build the checker libraries (test infrastructure, never the product).

* ``oracle/liboracle.so``: the C restatements in ``oracle/*.c``.
* ``oracle/_ref/libpcc_ref.so``: the reference's own conduction sources
  (``src/flux/pcc/{conductionQ,conductionT,tridag}.c``) and
  ``oracle/_ref/libvf_ref.so``: its exact triangle-triangle view factor
  (``src/flux/view_factor/view_factor_narayanaswamy.c``), compiled directly
  with gcc from where they lie in the reference tree, when that tree is
  present (it is not on GPU machines, which then use ``liboracle.so``).
  The tree is ``$FLUXPY_REFERENCE``; unset, this recipe looks at the
  checkout's usual place in the build container, and without either it
  builds only ``liboracle.so`` and says so.

Both are compiled with ``-ffp-contract=off`` so that results do not depend on
FMA contraction (gcc contracts by default on aarch64).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REF_DIR = ORACLE_DIR / "_ref"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"
REF_PCC_LIB = REF_DIR / "libpcc_ref.so"
# the build container's read-only checkout of the reference
_CHECKOUT = Path("/root/reference")


def reference_root() -> Path | None:
    env = os.environ.get("FLUXPY_REFERENCE")
    if env:
        return Path(env)
    return _CHECKOUT if _CHECKOUT.is_dir() else None
REF_PCC_SOURCES = ["conductionQ.c", "conductionT.c", "tridag.c"]
REF_VF_LIB = REF_DIR / "libvf_ref.so"
REF_VF_SOURCES = ["view_factor_narayanaswamy.c"]

CFLAGS = ["-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math"]


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _cc(srcs, out: Path, extra=()) -> None:
    cmd = ["gcc", *CFLAGS, *extra, *map(str, srcs), "-o", str(out), "-lm", "-fopenmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"gcc failed:\n{' '.join(cmd)}\n{res.stderr}")


def build_oracle() -> Path:
    srcs = sorted(ORACLE_DIR.glob("*.c"))
    if _newer(ORACLE_LIB, srcs):
        _cc(srcs, ORACLE_LIB)
    return ORACLE_LIB


def build_ref() -> Path | None:
    root = reference_root()
    if root is None:
        print("oracle/build.py: no reference tree (set FLUXPY_REFERENCE); "
              "oracle/_ref not built", file=sys.stderr)
        return None
    pcc = root / "src" / "flux" / "pcc"
    srcs = [pcc / s for s in REF_PCC_SOURCES]
    if not all(s.exists() for s in srcs):
        print(f"oracle/build.py: {pcc} lacks {REF_PCC_SOURCES}; oracle/_ref not built",
              file=sys.stderr)
        return None
    REF_DIR.mkdir(exist_ok=True)
    if _newer(REF_PCC_LIB, srcs):
        _cc(srcs, REF_PCC_LIB, extra=["-I", str(pcc)])
    vf = root / "src" / "flux" / "view_factor"
    vsrcs = [vf / s for s in REF_VF_SOURCES]
    if all(s.exists() for s in vsrcs) and _newer(REF_VF_LIB, vsrcs):
        _cc(vsrcs, REF_VF_LIB, extra=["-I", str(vf)])
    return REF_PCC_LIB


def build() -> None:
    build_oracle()
    build_ref()


if __name__ == "__main__":
    build()
    print(ORACLE_LIB, REF_PCC_LIB if REF_PCC_LIB.exists() else "(no reference tree)")
