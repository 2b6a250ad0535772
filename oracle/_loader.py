"""ctypes loader for the oracle's C restatements (oracle/liboracle.so) and,
when it was built, the reference's own C sources (oracle/_ref/)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

_libs: dict[str, C.CDLL] = {}


def oracle_lib() -> C.CDLL:
    if "oracle" not in _libs:
        path = _build.build_oracle()
        _libs["oracle"] = C.CDLL(str(path))
    return _libs["oracle"]


def ref_pcc_lib() -> C.CDLL | None:
    """The reference's conduction C sources compiled as-is, or None when the
    reference tree is not available (GPU machines)."""
    if "ref_pcc" not in _libs:
        path = _build.REF_PCC_LIB if _build.REF_PCC_LIB.exists() else _build.build_ref()
        if path is None or not Path(path).exists():
            return None
        _libs["ref_pcc"] = C.CDLL(str(path))
    return _libs["ref_pcc"]


def ref_vf_lib() -> C.CDLL | None:
    """The reference's exact triangle-triangle view factor compiled as-is
    (ff_narayanaswamy_impl), or None when the reference tree is not
    available."""
    if "ref_vf" not in _libs:
        if not _build.REF_VF_LIB.exists():
            _build.build_ref()
        if not _build.REF_VF_LIB.exists():
            return None
        lib = C.CDLL(str(_build.REF_VF_LIB))
        lib.ff_narayanaswamy_impl.restype = C.c_double
        lib.ff_narayanaswamy_impl.argtypes = [C.c_void_p, C.c_void_p]
        _libs["ref_vf"] = lib
    return _libs["ref_vf"]
