"""ORACLE — CPU visibility and form factors (test infrastructure).

Python entry points over oracle/vis_oracle.c, which restates the Embree and
CGAL backends' semantics (src/flux/shape.py:349-421,
src/flux/cgal/aabb_wrapper.cpp:64-108) and get_form_factor_matrix
(src/flux/form_factors.py:11-72), plus numpy restatements of the facet
geometry (shape.py:16-45).  Semantics: 0 = Embree, 1 = CGAL.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse

from ._loader import oracle_lib

EMBREE, CGAL = 0, 1
DEFAULT_EPS = 1e-5  # src/flux/config.py:2

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_l = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = oracle_lib()
        L.oracle_bvh_build.argtypes = [_d, C.c_longlong, _l, C.c_longlong]
        L.oracle_bvh_build.restype = C.c_void_p
        L.oracle_bvh_free.argtypes = [C.c_void_p]
        L.oracle_visibility.argtypes = [C.c_void_p, _d, _l, C.c_longlong, _l, C.c_longlong, C.c_int,
                                        C.c_int, _u8, C.c_void_p]
        L.oracle_occluded.argtypes = [C.c_void_p, _d, _d, _l, C.c_longlong, _d, C.c_longlong,
                                      C.c_int, C.c_int, _u8]
        L.oracle_ff_dense.argtypes = [C.c_void_p, _d, _d, _d, _l, C.c_longlong, _l, C.c_longlong,
                                      C.c_double, C.c_int, _d, C.c_void_p]
        L.oracle_ff_rows.argtypes = [C.c_void_p, _d, _d, _d, _l, C.c_longlong, C.c_double, C.c_int,
                                     _d]
        _lib = L
    return _lib


def geometry(V, F):
    """P, N, A exactly as src/flux/shape.py:16-45 computes them."""
    VF = V[F]
    P = VF.mean(axis=1)
    V0 = VF[:, 0, :]
    Cr = np.cross(VF[:, 1, :] - V0, VF[:, 2, :] - V0)
    Cn = np.sqrt(np.sum(Cr**2, axis=1))
    return P, Cr / Cn.reshape(Cr.shape[0], 1), Cn / 2


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


class Scene:
    """CPU ray-casting scene over a triangle mesh (FP32 and FP64 copies)."""

    def __init__(self, V, F):
        self.V = _c(V)
        self.F = _c(F, np.int64)
        self.nf = self.F.shape[0]
        self._h = lib().oracle_bvh_build(self.V, self.V.shape[0], self.F, self.nf)

    def __del__(self):
        try:
            if self._h:
                lib().oracle_bvh_free(self._h)
        except Exception:
            pass

    def visibility(self, P, I, J, sem=EMBREE, paired=False, near_edge=False):
        I = _c(np.atleast_1d(I), np.int64)
        J = _c(np.atleast_1d(J), np.int64)
        m, n = I.size, J.size
        out = np.zeros(m if paired else m * n, np.uint8)
        ne = np.zeros_like(out) if near_edge else None
        lib().oracle_visibility(self._h, _c(P), I, m, J, n, int(paired), sem, out,
                                ne.ctypes.data if ne is not None else None)
        vis = out.astype(bool) if paired else out.reshape(m, n).astype(bool)
        if near_edge:
            return vis, (ne.astype(bool) if paired else ne.reshape(m, n).astype(bool))
        return vis

    def occluded(self, P, N, I, D, sem=EMBREE):
        I = _c(np.atleast_1d(I), np.int64)
        D = _c(D)
        if D.ndim == 1:
            out = np.zeros(I.size, np.uint8)
            lib().oracle_occluded(self._h, _c(P), _c(N), I, I.size, D, 1, 0, sem, out)
            return out.astype(bool)
        out = np.zeros(I.size * D.shape[0], np.uint8)
        lib().oracle_occluded(self._h, _c(P), _c(N), I, I.size, D, D.shape[0], 0, sem, out)
        return out.reshape(I.size, D.shape[0]).astype(bool)

    def ff_dense(self, P, N, A, I=None, J=None, eps=DEFAULT_EPS, sem=EMBREE, info=False):
        """Dense F[I][:, J] as get_form_factor_matrix defines it."""
        I = np.arange(self.nf) if I is None else np.asarray(I)
        J = np.arange(self.nf) if J is None else np.asarray(J)
        I = _c(I, np.int64)
        J = _c(J, np.int64)
        out = np.zeros((I.size, J.size))
        inf = np.zeros((I.size, J.size), np.uint8) if info else None
        lib().oracle_ff_dense(self._h, _c(P), _c(N), _c(A), I, I.size, J, J.size, float(eps), sem,
                              out, inf.ctypes.data if inf is not None else None)
        return (out, inf) if info else out

    def ff_csr(self, P, N, A, I=None, J=None, eps=DEFAULT_EPS, sem=EMBREE):
        return scipy.sparse.csr_matrix(self.ff_dense(P, N, A, I, J, eps, sem))

    def ff_rows(self, P, N, A, I, eps=DEFAULT_EPS, sem=EMBREE):
        """Exact rows F[I, :] (all columns), for sampled-row checks."""
        I = _c(np.atleast_1d(I), np.int64)
        out = np.zeros((I.size, self.nf))
        lib().oracle_ff_rows(self._h, _c(P), _c(N), _c(A), I, I.size, float(eps), sem, out)
        return out
