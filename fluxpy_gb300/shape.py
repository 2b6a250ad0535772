"""Triangle-mesh shape models on the GPU: drop-in for ``flux.shape``.

The public surface follows src/flux/shape.py: ``get_centroids``,
``get_surface_normals_and_face_areas`` etc., ``TrimeshShapeModel`` with
``P, N, A, V, F``, ``get_visibility``, ``get_visibility_1_to_N``,
``get_visibility_matrix``, ``is_occluded``, ``get_direct_irradiance``,
``intersect1`` and pickling through ``__reduce__``; and the two backends
``CgalTrimeshShapeModel`` / ``EmbreeTrimeshShapeModel``.

Both backends run on one device-side linear BVH (libfluxgb ``fgb_bvh_*``)
and differ only in ray semantics (visibility.cuh): Embree's FP32 rays with an
absolute 1e-3 origin offset, or CGAL's FP64 rays from the face centroid with
the source face skipped.

``P, N, A`` are host numpy arrays, as in the reference; callers may edit them
in place (the reference tests flip normals after construction), so the device
copies are refreshed whenever the host arrays change.
"""
from __future__ import annotations

from abc import ABC

import numpy as np
import torch

from . import _lib

EMBREE, CGAL = 0, 1
use1M = True


def get_centroids(V, F):
    return V[F].mean(axis=1)


def get_cross_products(V, F):
    V0 = V[F][:, 0, :]
    return np.cross(V[F][:, 1, :] - V0, V[F][:, 2, :] - V0)


def get_face_areas(V, F):
    C = get_cross_products(V, F)
    return np.sqrt(np.sum(C**2, axis=1)) / 2


def get_surface_normals(V, F):
    C = get_cross_products(V, F)
    C_norms = np.sqrt(np.sum(C**2, axis=1))
    return C / C_norms.reshape(C.shape[0], 1)


def get_surface_normals_and_face_areas(V, F):
    C = get_cross_products(V, F)
    C_norms = np.sqrt(np.sum(C**2, axis=1))
    return C / C_norms.reshape(C.shape[0], 1), C_norms / 2


_FN = {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}
_TDT = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32}


def device_facet_geometry(V_d: torch.Tensor, F_d: torch.Tensor):
    """P, N, A of a device mesh (bit-identical to shape.py:16-45)."""
    nf = F_d.shape[0]
    P = torch.empty((nf, 3), dtype=V_d.dtype, device=V_d.device)
    N = torch.empty_like(P)
    A = torch.empty((nf,), dtype=V_d.dtype, device=V_d.device)
    flags = torch.zeros(1, dtype=torch.int32, device=V_d.device)
    sfx = "f64" if V_d.dtype == torch.float64 else "f32"
    _lib.call(f"fgb_facet_geometry_{sfx}", _lib.ptr(V_d), V_d.shape[0], _lib.ptr(F_d), nf,
              _lib.ptr(P), _lib.ptr(N), _lib.ptr(A), _lib.ptr(flags), _lib.stream_handle())
    if int(flags.item()) & _lib.FLAG_INDEX_RANGE:
        raise ValueError("face indices out of range of the vertex array")
    return P, N, A


class DeviceBVH:
    """Owner of a libfluxgb BVH handle."""

    def __init__(self, V_d: torch.Tensor, F_d: torch.Tensor, keep_f64: bool):
        import ctypes
        self._h = ctypes.c_void_p()
        flags = torch.zeros(1, dtype=torch.int32, device=V_d.device)
        sfx = "f64" if V_d.dtype == torch.float64 else "f32"
        _lib.call(f"fgb_bvh_build_{sfx}", _lib.ptr(V_d), V_d.shape[0], _lib.ptr(F_d),
                  F_d.shape[0], int(keep_f64), ctypes.byref(self._h), _lib.ptr(flags),
                  _lib.stream_handle())
        if int(flags.item()) & _lib.FLAG_INDEX_RANGE:
            raise ValueError("face indices out of range of the vertex array")

    @property
    def handle(self):
        return self._h.value

    def nbytes(self) -> int:
        import ctypes
        n, b = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.call("fgb_bvh_info", self._h.value, ctypes.byref(n), ctypes.byref(b))
        return b.value

    def __del__(self):
        try:
            if self._h and self._h.value:
                _lib.lib().fgb_bvh_free(self._h.value)
                self._h = None
        except Exception:
            pass


class ShapeModel(ABC):
    pass


class TrimeshShapeModel(ShapeModel):
    """A shape model consisting of a single triangle mesh (shape.py:52)."""

    _semantics = EMBREE

    def __init__(self, V, F, N=None, P=None, A=None):
        if type(self) == TrimeshShapeModel:
            raise RuntimeError("tried to instantiate TrimeshShapeModel directly")
        self.dtype = V.dtype
        self.V = V
        self.F = F

        if self.dtype not in _FN:
            raise RuntimeError(f"unsupported dtype {self.dtype}")
        dev = _lib.require_cuda()
        self._device = dev
        self._V_d = torch.as_tensor(np.ascontiguousarray(V), device=dev)
        self._F_d = torch.as_tensor(np.ascontiguousarray(F, dtype=np.int64), device=dev)
        if N is not None and N.shape[0] != F.shape[0] and A is None:
            raise Exception(
                'must pass same number of surface normals as faces (got ' +
                '%d faces and %d normals' % (F.shape[0], N.shape[0]))
        Pd, Nd, Ad = device_facet_geometry(self._V_d, self._F_d)
        # the reference always recomputes the centroids (shape.py:104)
        self.P = Pd.cpu().numpy()
        self.N = Nd.cpu().numpy() if N is None else N
        self.A = Ad.cpu().numpy() if A is None else A
        assert self.P.dtype == self.dtype
        assert self.N.dtype == self.dtype
        assert self.A.dtype == self.dtype
        self._geom_cache = None
        self._make_scene()

    # -- scene ----------------------------------------------------------
    def _make_scene(self):
        self._bvh = DeviceBVH(self._V_d, self._F_d, keep_f64=(self._semantics == CGAL))

    def __reduce__(self):
        return (self.__class__, (self.V, self.F, self.N, self.P, self.A))

    def __repr__(self):
        return 'a TrimeshShapeModel with %d vertices and %d faces' % (
            self.num_verts, self.num_faces)

    @property
    def num_faces(self):
        return self.P.shape[0]

    @property
    def num_verts(self):
        return self.V.shape[0]

    @property
    def bvh(self) -> DeviceBVH:
        return self._bvh

    @property
    def semantics(self) -> int:
        return self._semantics

    def device_geometry(self):
        """(P, N, A) as device tensors in the shape dtype, refreshed if the
        host arrays were modified since the last call."""
        c = self._geom_cache
        host = (self.P, self.N, self.A)
        if c is not None and all(h is ch and np.array_equal(h, hc)
                                 for h, ch, hc in zip(host, c[0], c[1])):
            return c[2]
        tdt = _TDT[np.dtype(self.dtype)]
        dev = tuple(torch.as_tensor(np.ascontiguousarray(h), dtype=tdt, device=self._device)
                    for h in host)
        self._geom_cache = (host, tuple(h.copy() for h in host), dev)
        return dev

    # -- queries ----------------------------------------------------------
    def intersect1(self, x, d):
        '''Trace a single ray from x along d; return (i, hit point) or None.'''
        return self._intersect1(x, d)

    def get_visibility(self, I, J, oriented=False):
        vis = self._get_visibility(I, J)
        if oriented:
            I_, J_ = np.where(vis)
            I_arr = np.asarray(I)[I_] if np.ndim(I) else I_
            J_arr = np.asarray(J)[J_]
            mask = ((self.P[J_arr] - self.P[I_arr]) * self.N[I_arr]).sum(1) <= 0
            vis[I_[mask], J_[mask]] = False
        return vis

    def get_visibility_1_to_N(self, i, J, oriented=False):
        return self.get_visibility([i], J, oriented).ravel()

    def get_visibility_matrix(self, oriented=False):
        I = np.arange(self.num_faces, dtype=np.uintp)
        return self.get_visibility(I, I, oriented)

    def is_occluded(self, I, D):
        return self._is_occluded(I, D)

    def get_direct_irradiance(self, F0, Dsun, basemesh=None, eps=None):
        '''Insolation from the sun (shape.py:190-244).'''
        if basemesh is None:
            basemesh = self
        if Dsun.ndim == 1:
            I = ~basemesh.is_occluded(np.arange(self.num_faces), Dsun)
            E = np.zeros(self.num_faces, dtype=self.dtype)
            E[I] = F0 * np.maximum(0, self.N[I] @ Dsun)
        elif (Dsun.ndim == 2) & (Dsun.shape[0] == self.num_faces):
            if Dsun.shape[1] != 3:
                raise ValueError('need Dsun.shape[1] == 3 if Dsun.ndim == 2')
            I = ~basemesh.is_occluded(np.arange(self.num_faces), Dsun)
            E = np.zeros(self.num_faces, dtype=self.dtype)
            E[I] = F0 * np.maximum(0, (self.N[I] * Dsun[I]).sum(1))
        elif Dsun.ndim == 2:
            if Dsun.shape[1] != 3:
                raise ValueError('need Dsun.shape[1] == 3 if Dsun.ndim == 2')
            I = ~basemesh._is_occluded_all_dirs(np.arange(self.num_faces), Dsun)
            E = self.N @ Dsun.T
            E = np.where(I, E, 0)
            E = np.mean(F0) * np.maximum(0, np.sum(E, axis=1) / Dsun.shape[0])
        else:
            raise RuntimeError('Dsun.ndim > 2 not implemented yet')
        return E

    def get_direct_irradiance_batch(self, F0, Dsun, out_dtype=None, device_out=True):
        """Insolation for K sun directions at once: E of shape (num_faces, K)
        with E[:, k] == get_direct_irradiance(F0[k], Dsun[k]) (one FP32/FP64
        ray per facet and direction on the GPU).  Returns a device tensor
        unless device_out is False."""
        Dsun = np.atleast_2d(np.asarray(Dsun, dtype=self.dtype))
        K = Dsun.shape[0]
        F0 = np.broadcast_to(np.asarray(F0, dtype=self.dtype), (K,)).copy()
        P, N, _ = self.device_geometry()
        tdt = _TDT[np.dtype(self.dtype)]
        D_d = torch.as_tensor(Dsun, dtype=tdt, device=self._device)
        F0_d = torch.as_tensor(F0, dtype=tdt, device=self._device)
        odt = tdt if out_dtype is None else out_dtype
        E = torch.empty((self.num_faces, K), dtype=odt, device=self._device)
        flags = torch.zeros(1, dtype=torch.int32, device=self._device)
        sfx = _FN[np.dtype(self.dtype)]
        if odt == torch.float32 and tdt == torch.float64:
            fn = "fgb_direct_irradiance_f64_to_f32"
        elif odt == tdt:
            fn = f"fgb_direct_irradiance_{sfx}"
        else:
            raise ValueError("unsupported output dtype")
        _lib.call(fn, self._bvh.handle, _lib.ptr(P), _lib.ptr(N), self.num_faces, _lib.ptr(D_d), K,
                  _lib.ptr(F0_d), self._semantics, _lib.ptr(E), _lib.ptr(flags),
                  _lib.stream_handle())
        self._check_flags(flags)
        return E if device_out else E.cpu().numpy()

    # -- backend calls --------------------------------------------------
    def _check_flags(self, flags):
        f = int(flags.item())
        if f & _lib.FLAG_STACK_OVERFLOW:
            raise RuntimeError("BVH traversal stack overflow")
        if f & _lib.FLAG_INDEX_RANGE:
            raise IndexError("facet index out of range")

    def _index(self, I):
        a = np.asarray(I)
        if a.ndim == 0:
            a = a.reshape(1)
        return torch.as_tensor(a.astype(np.int64), device=self._device)

    def _get_visibility(self, I, J):
        I_d, J_d = self._index(I), self._index(J)
        m, n = I_d.numel(), J_d.numel()
        P, _, _ = self.device_geometry()
        vis = torch.empty((m, n), dtype=torch.uint8, device=self._device)
        flags = torch.zeros(1, dtype=torch.int32, device=self._device)
        _lib.call(f"fgb_visibility_{_FN[np.dtype(self.dtype)]}", self._bvh.handle, _lib.ptr(P),
                  self.num_faces, _lib.ptr(I_d), m, _lib.ptr(J_d), n, 0, self._semantics,
                  _lib.ptr(vis), None, _lib.ptr(flags), _lib.stream_handle())
        self._check_flags(flags)
        return vis.cpu().numpy().astype(bool)

    def get_visibility_pairs(self, I, J, near_edge=False):
        """Visibility of the pairs (I[k], J[k]) (device-side extension)."""
        I_d, J_d = self._index(I), self._index(J)
        m = I_d.numel()
        if J_d.numel() != m:
            raise ValueError("I and J must have the same length")
        P, _, _ = self.device_geometry()
        vis = torch.empty(m, dtype=torch.uint8, device=self._device)
        ne = torch.empty(m, dtype=torch.uint8, device=self._device) if near_edge else None
        flags = torch.zeros(1, dtype=torch.int32, device=self._device)
        _lib.call(f"fgb_visibility_{_FN[np.dtype(self.dtype)]}", self._bvh.handle, _lib.ptr(P),
                  self.num_faces, _lib.ptr(I_d), m, _lib.ptr(J_d), m, 1, self._semantics,
                  _lib.ptr(vis), _lib.ptr(ne), _lib.ptr(flags), _lib.stream_handle())
        self._check_flags(flags)
        v = vis.cpu().numpy().astype(bool)
        return (v, ne.cpu().numpy().astype(bool)) if near_edge else v

    def _occluded_call(self, I, D, per_facet):
        I_d = self._index(I)
        m = I_d.numel()
        P, N, _ = self.device_geometry()
        tdt = _TDT[np.dtype(self.dtype)]
        D_d = torch.as_tensor(np.ascontiguousarray(np.atleast_2d(D), dtype=self.dtype),
                              dtype=tdt, device=self._device)
        ndirs = D_d.shape[0]
        out = torch.empty(m if per_facet else m * ndirs, dtype=torch.uint8, device=self._device)
        flags = torch.zeros(1, dtype=torch.int32, device=self._device)
        _lib.call(f"fgb_occluded_{_FN[np.dtype(self.dtype)]}", self._bvh.handle, _lib.ptr(P),
                  _lib.ptr(N), self.num_faces, _lib.ptr(I_d), m, _lib.ptr(D_d), ndirs,
                  int(per_facet), self._semantics, _lib.ptr(out), _lib.ptr(flags),
                  _lib.stream_handle())
        self._check_flags(flags)
        o = out.cpu().numpy().astype(bool)
        return o if per_facet else o.reshape(m, ndirs)

    def _is_occluded_all_dirs(self, I, D):
        return self._occluded_call(I, D, per_facet=False)


class CgalTrimeshShapeModel(TrimeshShapeModel):
    """CGAL-semantics backend (shape.py:261-292): FP64 rays from the face
    centroid, source face skipped, first hit decides."""

    _semantics = CGAL

    def _intersect1(self, x, d):
        X = torch.as_tensor(np.asarray(x, dtype=np.float64).reshape(1, 3), device=self._device)
        D = torch.as_tensor(np.asarray(d, dtype=np.float64).reshape(1, 3), device=self._device)
        hit = torch.empty(1, dtype=torch.int64, device=self._device)
        xt = torch.empty((1, 3), dtype=torch.float64, device=self._device)
        flags = torch.zeros(1, dtype=torch.int32, device=self._device)
        _lib.call("fgb_intersect1_f64", self._bvh.handle, _lib.ptr(X), _lib.ptr(D), 1,
                  _lib.ptr(hit), _lib.ptr(xt), _lib.ptr(flags), _lib.stream_handle())
        self._check_flags(flags)
        i = int(hit.item())
        if i >= 0:
            return i, xt.cpu().numpy()[0]
        return None

    def _is_occluded(self, I, D):
        D = np.asarray(D)
        if D.ndim == 1:
            return self._occluded_call(I, D, per_facet=False)[:, 0]
        elif D.ndim == 2:
            return self._occluded_call(I, D, per_facet=False)
        raise ValueError('D.ndim should be 1 or 2')


class EmbreeTrimeshShapeModel(TrimeshShapeModel):
    """Embree-semantics backend (shape.py:295-421): FP32 scene and rays,
    absolute 1e-3 origin offset."""

    _semantics = EMBREE

    def _intersect1(self, x, d):
        raise RuntimeError('intersect1 no implemented for EmbreeTrimeshShapeModel')

    def _is_occluded(self, I, D):
        D = np.asarray(D)
        if D.ndim != 1 and D.ndim != 2:
            raise ValueError('D.ndim should be 1 or 2')
        if D.ndim == 1:
            return self._occluded_call(I, D, per_facet=False)[:, 0]
        m = np.size(I)
        if D.shape[0] == m:
            return self._occluded_call(I, D, per_facet=True)
        if D.shape[0] == 1:
            return self._occluded_call(I, D, per_facet=False)[:, 0]
        raise ValueError(f'could not broadcast {D.shape[0]} directions to {m} rays')


trimesh_shape_models = [
    CgalTrimeshShapeModel,
    EmbreeTrimeshShapeModel,
]
