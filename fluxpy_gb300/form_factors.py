"""Form-factor assembly on the GPU: drop-in for ``flux.form_factors``.

``get_form_factor_matrix(shape_model, I=None, J=None, eps=None)`` returns the
same scipy CSR matrix as src/flux/form_factors.py:11-72: entry (r, c) is
F(I[r], J[c]) = cos(theta_i) cos(theta_j) A_j / (pi r^2) for pairs that pass
the absolute orientation threshold ``eps`` (config.DEFAULT_EPS) and are
visible under the shape model's backend semantics; column indices are
positions in J.  The pairs are evaluated by the fused pair kernel
(libfluxgb ``fgb_ff_count_*`` / ``fgb_ff_fill_*``, one visibility ray per
kept pair) instead of a Python loop over rows.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse
import torch

from . import _lib, config

_SFX = {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}


class TileCSR:
    """Device CSR produced by the pair kernel for a list of tiles: rows of
    tile t are [row_off[t], row_off[t+1]) of ``indptr``; column indices are
    local to the tile."""

    def __init__(self, indptr, indices, data, row_off, kept_pairs, near_edge_pairs, bits=None,
                 word_off=None):
        self.indptr = indptr
        self.indices = indices
        self.data = data
        self.row_off = row_off
        self.kept_pairs = kept_pairs
        self.near_edge_pairs = near_edge_pairs
        self.bits = bits          # visible-pair bitmask (kept when asked for)
        self.word_off = word_off  # per-tile offsets into bits


def ff_tiles(shape_model, I_d, J_d, row0, nrows, col0, ncols, eps=None, keep_bits=False,
             out_dtype=None) -> TileCSR:
    """Evaluate the form factors of a list of tiles on the device.

    I_d, J_d: int64 device tensors of facet ids; tile t covers rows
    I_d[row0[t]:row0[t]+nrows[t]] and columns J_d[col0[t]:col0[t]+ncols[t]]
    (row0 etc. are int64 numpy arrays)."""
    if eps is None:
        eps = config.DEFAULT_EPS
    dev = I_d.device
    P, N, A = shape_model.device_geometry()
    sfx = _SFX[np.dtype(shape_model.dtype)]
    row0 = np.asarray(row0, np.int64)
    nrows = np.asarray(nrows, np.int64)
    col0 = np.asarray(col0, np.int64)
    ncols = np.asarray(ncols, np.int64)
    T = row0.size
    wpr = (ncols + 31) // 32
    word_off = np.zeros(T + 1, np.int64)
    np.cumsum(nrows * wpr, out=word_off[1:])
    row_off = np.zeros(T + 1, np.int64)
    np.cumsum(nrows, out=row_off[1:])
    W, R = int(word_off[-1]), int(row_off[-1])

    def d(a):
        return torch.as_tensor(a, device=dev)

    t_row0, t_nrows, t_col0, t_ncols, t_woff, t_roff = map(d, (row0, nrows, col0, ncols, word_off,
                                                               row_off))
    bits = torch.empty(max(W, 1), dtype=torch.int32, device=dev)
    cnt = torch.zeros(max(R, 1), dtype=torch.int32, device=dev)
    stats = torch.zeros(2, dtype=torch.int64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = _lib.stream_handle()
    _lib.call(f"fgb_ff_count_{sfx}", shape_model.bvh.handle, _lib.ptr(P), _lib.ptr(N), _lib.ptr(A),
              _lib.ptr(I_d), _lib.ptr(J_d), _lib.ptr(t_row0), _lib.ptr(t_nrows), _lib.ptr(t_col0),
              _lib.ptr(t_ncols), _lib.ptr(t_woff), _lib.ptr(t_roff), T, W, float(eps),
              shape_model.semantics, _lib.ptr(bits), _lib.ptr(cnt), _lib.ptr(stats),
              _lib.ptr(flags), stream)
    indptr = torch.zeros(R + 1, dtype=torch.int64, device=dev)
    if R:
        torch.cumsum(cnt[:R].to(torch.int64), 0, out=indptr[1:])
    nnz = int(indptr[-1].item())
    if int(flags.item()) & _lib.FLAG_STACK_OVERFLOW:
        raise RuntimeError("BVH traversal stack overflow")
    tdt = P.dtype if out_dtype is None else out_dtype
    indices = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    data = torch.empty(max(nnz, 1), dtype=tdt, device=dev)
    fill = f"fgb_ff_fill_{sfx}"
    if tdt != P.dtype:
        if not (P.dtype == torch.float64 and tdt == torch.float32):
            raise ValueError("unsupported output dtype")
        fill = "fgb_ff_fill_f64_to_f32"
    _lib.call(fill, _lib.ptr(P), _lib.ptr(N), _lib.ptr(A), _lib.ptr(I_d),
              _lib.ptr(J_d), _lib.ptr(t_row0), _lib.ptr(t_nrows), _lib.ptr(t_col0),
              _lib.ptr(t_ncols), _lib.ptr(t_woff), _lib.ptr(t_roff), T, R, _lib.ptr(bits),
              _lib.ptr(indptr), _lib.ptr(indices), _lib.ptr(data), stream)
    st = stats.cpu().numpy()
    return TileCSR(indptr, indices[:nnz], data[:nnz], row_off, int(st[0]), int(st[1]),
                   bits if keep_bits else None, word_off if keep_bits else None)


def _as_index(x, n):
    if x is None:
        return np.arange(n, dtype=np.int64)
    return np.asarray(x).astype(np.int64).reshape(-1)


def exact_adjacent_fix(shape_model, I_d, J_d, t: TileCSR) -> int:
    """Replace the entries of a one-tile device CSR (rows I_d, columns J_d)
    whose two facets share a vertex by the exact triangle view factor
    (libfluxgb ``fgb_ff_adjacent_fix_f64``); returns how many changed."""
    dev = I_d.device
    if t.data.dtype != torch.float64:
        raise ValueError("the exact adjacent-facet correction needs an FP64 matrix")
    V = torch.as_tensor(np.asarray(shape_model.V, np.float64), device=dev)
    F = torch.as_tensor(np.asarray(shape_model.F, np.int64), device=dev)
    fixed = torch.zeros(1, dtype=torch.int64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("fgb_ff_adjacent_fix_f64", _lib.ptr(V), _lib.ptr(F), _lib.ptr(I_d), _lib.ptr(J_d),
              int(I_d.numel()), _lib.ptr(t.indptr), _lib.ptr(t.indices), _lib.ptr(t.data),
              _lib.ptr(fixed), _lib.ptr(flags), _lib.stream_handle())
    if int(flags.item()) & _lib.FLAG_NONFINITE_OUT:
        raise RuntimeError("non-finite exact view factor")
    return int(fixed.item())


def get_form_factor_matrix(shape_model, I=None, J=None, eps=None, exact_adjacent=False):
    """scipy CSR of F[I][:, J] (src/flux/form_factors.py:11-72).

    exact_adjacent (an addition): entries whose two facets share a vertex,
    where the midpoint rule is least accurate, are replaced by the exact
    view factor of the two triangles (the closed form that the reference
    offers separately as flux.view_factor.ff_narayanaswamy); FP64 shape
    models only."""
    n_faces = shape_model.P.shape[0]
    if shape_model.dtype not in _SFX:
        raise RuntimeError(f'unsupported dtype {shape_model.dtype}')
    I = _as_index(I, n_faces)
    J = _as_index(J, n_faces)
    m, n = I.size, J.size
    if m == 0 or n == 0:
        return scipy.sparse.csr_matrix((m, n), dtype=shape_model.dtype)
    dev = shape_model._device
    I_d = torch.as_tensor(I, device=dev)
    J_d = torch.as_tensor(J, device=dev)
    t = ff_tiles(shape_model, I_d, J_d, [0], [m], [0], [n], eps)
    if exact_adjacent:
        exact_adjacent_fix(shape_model, I_d, J_d, t)
    data = t.data.cpu().numpy()
    indices = t.indices.cpu().numpy()
    indptr = t.indptr.cpu().numpy()
    return scipy.sparse.csr_matrix((data, indices, indptr), shape=(m, n))


def get_form_factor_matrix_device(shape_model, I=None, J=None, eps=None) -> TileCSR:
    """Like get_form_factor_matrix, but the CSR stays on the device."""
    n_faces = shape_model.P.shape[0]
    I = _as_index(I, n_faces)
    J = _as_index(J, n_faces)
    dev = shape_model._device
    return ff_tiles(shape_model, torch.as_tensor(I, device=dev), torch.as_tensor(J, device=dev),
                    [0], [I.size], [0], [J.size], eps)
