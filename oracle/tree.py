"""ORACLE — octree / quadtree partition rule (test infrastructure).

Restates get_octant_order (src/flux/octree.py:5-18) and get_quadrant_order
(src/flux/quadtree.py:5-18): split a point set about the midpoint of its
bounding box, coordinate <= midpoint going to the low side, children in
itertools.product([low, high], repeat=d) order, each child listing the
positions of its points in ascending order.
"""
import itertools as it

import numpy as np


def orthant_order(X):
    X = np.asarray(X, dtype=np.float64)
    d = X.shape[1]
    mid = (X.min(axis=0) + X.max(axis=0)) / 2
    out = []
    for sides in it.product([False, True], repeat=d):
        sel = np.ones(X.shape[0], dtype=bool)
        for a, high in enumerate(sides):
            sel &= (X[:, a] > mid[a]) if high else (X[:, a] <= mid[a])
        out.append(np.flatnonzero(sel))
    return out
