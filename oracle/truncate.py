"""ORACLE — rank truncation of a low-rank block on the CPU (test
infrastructure, never the product).

Restates the reference's truncation rule, src/flux/linalg.py:20-51
(estimate_rank, as FormFactor2dTreeBlock._get_svd_block applies it,
src/flux/compressed_form_factors.py:388-405): the singular values of the
block in decreasing order, rank r = the first i with sigma_i / sigma_0 <= tol
(every value kept when none is), the block kept as its leading r singular
triplets.  The reference finds the singular values with ARPACK (svds from a
random start, k = 40, 80, ...); here with a dense FP64 SVD of the block
U V^T, which gives the same values to working precision.
"""
import numpy as np


def truncation_rank(s, tol):
    """r = the first index with s[i] / s[0] <= tol (len(s) when none)."""
    s = np.asarray(s, np.float64)
    if s.size == 0 or s[0] == 0:
        return 0
    below = np.flatnonzero(s / s[0] <= tol)
    return int(below[0]) if below.size else int(s.size)


def truncate(U, V, tol):
    """Block U V^T (U: m x k, V: n x k) -> (singular values, r, U_r V_r^T)."""
    A = np.asarray(U, np.float64) @ np.asarray(V, np.float64).T
    Uf, s, Vt = np.linalg.svd(A, full_matrices=False)
    r = truncation_rank(s, tol)
    return s, r, (Uf[:, :r] * s[:r]) @ Vt[:r]
