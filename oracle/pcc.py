"""ORACLE — PCC 1-D conduction on the CPU (test infrastructure).

Python entry points over oracle/pcc_oracle.c, which restates
src/flux/pcc/conductionQ.c:10-186, conductionT.c:4-88 and tridag.c:5-34
with the facet loop of src/flux/thermal.pyx:249-286.  ``ref_step_q`` runs the
reference's own ``conductionQ`` (oracle/_ref) when it is available.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._loader import oracle_lib, ref_pcc_lib

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def _setup(lib):
    lib.oracle_pcc_step_q.argtypes = [C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp,
                                      _dp, _dp, _dp]
    lib.oracle_pcc_step_q.restype = C.c_int
    lib.oracle_pcc_step_t.argtypes = [C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp,
                                      _dp, _dp]
    lib.oracle_pcc_step_t.restype = C.c_int
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _setup(oracle_lib())
    return _lib


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def step_q(z, dt, Qprev, X, T, ti, rhoc, emiss, Fgeotherm):
    """One conductionQ step for every facet; T (num_faces, nz+1) float64
    C-contiguous is updated in place.  Returns Fsurf."""
    assert T.dtype == np.float64 and T.flags.c_contiguous
    n, w = T.shape
    Fsurf = np.empty(n)
    st = lib().oracle_pcc_step_q(n, w - 1, _c(z), float(dt), _c(Qprev), _c(X), T, _c(ti),
                                 _c(rhoc), _c(emiss), _c(Fgeotherm), Fsurf)
    if st:
        raise RuntimeError("tridag failed")
    return Fsurf


def step_t(z, dt, Tsprev, X, T, ti, rhoc, Fgeotherm):
    assert T.dtype == np.float64 and T.flags.c_contiguous
    n, w = T.shape
    Fsurf = np.empty(n)
    st = lib().oracle_pcc_step_t(n, w - 1, _c(z), float(dt), _c(Tsprev), _c(X), T, _c(ti),
                                 _c(rhoc), _c(Fgeotherm), Fsurf)
    if st:
        raise RuntimeError("tridag failed")
    return Fsurf


def ref_step_q(z, dt, Qprev, X, T, ti, rhoc, emiss, Fgeotherm):
    """Same as step_q through the reference's own conductionQ (oracle/_ref),
    or None when it is not available."""
    ref = ref_pcc_lib()
    if ref is None:
        return None
    f = ref.conductionQ
    dptr = C.POINTER(C.c_double)
    f.argtypes = [C.c_int, dptr, C.c_double, C.c_double, C.c_double, dptr, dptr, dptr,
                  C.c_double, C.c_double, dptr]
    f.restype = None
    n, w = T.shape
    z, ti, rhoc = _c(z), _c(ti), _c(rhoc)
    Fsurf = np.empty(n)
    for i in range(n):
        row = T[i]
        f(w - 1, z.ctypes.data_as(dptr), float(dt), float(Qprev[i]), float(X[i]),
          row.ctypes.data_as(dptr), ti.ctypes.data_as(dptr), rhoc.ctypes.data_as(dptr),
          float(emiss[i]), float(Fgeotherm[i]), Fsurf[i:].ctypes.data_as(dptr))
    return Fsurf
