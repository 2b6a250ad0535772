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
