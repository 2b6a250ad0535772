"""CPU: libfluxgb.so loads and exports every entry point include/fluxgb.h
declares (no compute calls without a GPU)."""
import ctypes
import re
from pathlib import Path

from fluxpy_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "fluxgb.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "fgb_last_error" in syms and len(syms) > 10


def test_library_exports_all_declared_symbols():
    assert _lib.LIB_PATH.exists(), "build libfluxgb.so first"
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_table_matches_header():
    syms = set(declared_symbols())
    assert set(_lib.SIGNATURES) <= syms
    assert syms <= set(_lib.SIGNATURES), sorted(syms - set(_lib.SIGNATURES))


def test_version_and_error_strings():
    lib = _lib.lib()
    assert lib.fgb_version().decode().startswith("fluxgb")
    assert isinstance(lib.fgb_last_error().decode(), str)


def test_status_codes_map_to_the_reference_exception_types():
    import pytest
    _lib.check(_lib.FGB_OK)
    with pytest.raises(ValueError):
        _lib.check(_lib.FGB_BAD_ARG, "fgb_x")
    for st in (_lib.FGB_NONFINITE, _lib.FGB_ZERO_PIVOT, _lib.FGB_CUDA_ERR,
               _lib.FGB_DEVICE_TIMEOUT, _lib.FGB_NO_MEMORY):
        with pytest.raises(RuntimeError) as e:
            _lib.check(st, "fgb_x")
        assert isinstance(e.value, _lib.FluxGBError) and e.value.status == st


def test_no_cpu_fallback_without_a_device(monkeypatch):
    import pytest
    import torch
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.require_cuda()
