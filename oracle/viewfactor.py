"""ORACLE — view factor between two triangles on the CPU (test
infrastructure, never the product).

The definition the reference's closed form evaluates
(src/flux/view_factor/view_factor_narayanaswamy.c:338-494, Narayanaswamy
2015): F_AB = |(1 / area_A) int_A int_B cos(t_A) cos(t_B) / (pi r^2) dB dA|
with signed cosines (the contour-integral form counts a pair of points
that face away from each other negatively; for two triangles that face
each other it is the view factor), computed here by brute-force
quadrature: each triangle split into 4^level similar sub-triangles, one
point per sub-triangle (its centroid), so the error falls as the square of
the sub-triangle size for separated triangles.  ``ff_ref`` calls the
reference's own C compiled under oracle/_ref when it is available.
"""
import ctypes as C

import numpy as np

from ._loader import ref_vf_lib


def _subdivide(T, level):
    """Centroids and areas of the 4^level sub-triangles of T (3 x 3)."""
    tris = np.asarray(T, np.float64)[None]
    for _ in range(level):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
        tris = np.concatenate([np.stack(t, 1) for t in
                               ((a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca))])
    cen = tris.mean(1)
    area = 0.5 * np.linalg.norm(np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]), axis=1)
    return cen, area


def ff_quadrature(T1, T2, level=5):
    """View factor of triangle T1 towards T2 (vertices as rows), the
    normals from the vertex order ((v1 - v0) x (v2 - v0))."""
    T1, T2 = np.asarray(T1, np.float64), np.asarray(T2, np.float64)
    n1 = np.cross(T1[1] - T1[0], T1[2] - T1[0])
    n2 = np.cross(T2[1] - T2[0], T2[2] - T2[0])
    A1 = 0.5 * np.linalg.norm(n1)
    n1 /= np.linalg.norm(n1)
    n2 /= np.linalg.norm(n2)
    x, ax = _subdivide(T1, level)
    y, ay = _subdivide(T2, level)
    d = y[None, :, :] - x[:, None, :]
    r2 = np.sum(d * d, axis=2)
    c1 = d @ n1
    c2 = -(d @ n2)
    k = c1 * c2 / (np.pi * r2 * r2)
    return abs(float(ax @ k @ ay)) / A1


def ff_ref(T1, T2):
    """The reference's ff_narayanaswamy_impl, or None without oracle/_ref."""
    lib = ref_vf_lib()
    if lib is None:
        return None
    a = np.ascontiguousarray(T1, np.float64)
    b = np.ascontiguousarray(T2, np.float64)
    return float(lib.ff_narayanaswamy_impl(a.ctypes.data_as(C.c_void_p),
                                           b.ctypes.data_as(C.c_void_p)))
