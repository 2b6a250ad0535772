"""Hierarchical compressed form-factor matrix on the GPU: drop-in for
``flux.compressed_form_factors``.

Structure (src/flux/compressed_form_factors.py:285-386, 512-698): rows and
columns are split recursively into octants (``FormFactorOctreeBlock``) or
quadrants (``FormFactorQuadtreeBlock``, the default root) about the midpoint
of their bounding box, ``<=`` going to the low side (src/flux/octree.py:5-18,
quadtree.py:5-18); every block of that tree is a leaf (zero / dense / sparse
/ low-rank) or is subdivided again.

What differs from the reference, by design:
  * the reference assembles the full sparse matrix of every root block and
    picks, per block, the smallest of {CSR, ARPACK SVD, children}; here a
    block is low-rank when its two clusters are well separated
    (min(diam) <= eta * dist) and its adaptive cross approximation
    (libfluxgb ``fgb_aca_f64``, relative Frobenius tolerance ``aca_tol``,
    tol / 10 by default) converges under its rank cap; its factors are then
    truncated in FP64 to the singular values above ``tol`` times the
    largest (``fgb_recompress_f32``, the reference's SVD truncation rule,
    linalg.py:20-51); blocks below ``min_size`` entries, at
    ``max_depth``, or between leaf clusters are evaluated exactly by the
    fused pair kernel (``fgb_ff_count/fill``).  Only O(N log N) entries and
    rays are evaluated, not N^2.
  * the leaves live on the device in one flat layout (libfluxgb matvec.cu):
    the Python block tree (``_root._blocks`` etc.) is materialised lazily
    from it for introspection, with the reference's block classes and the
    reference's dense-vs-CSR choice by bytes and all-dense / all-sparse
    collapsing.
  * storage precision: ``dtype`` (default: the shape model's dtype, so FP64
    shape models reproduce the reference's FP64 products); FP32 and BF16
    copies are made for the fast paths.

Products: ``F @ x`` with numpy input returns numpy (the reference's
LinearOperator behaviour); with a CUDA tensor it stays on the device.
"""
from __future__ import annotations

import ctypes as C
import pickle

import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import torch

from . import _lib, config
from .form_factors import ff_tiles


# ------------------------------------------------------------------ tree --
class ClusterTree:
    """Recursive 2^d-ary partition of the facet centroids.

    ``perm`` lists facet ids in cluster order: every node is the contiguous
    range perm[start:start+size], grouped by its descendants.  The
    reference's index list of a node (its np.where order) is the same set in
    ascending id order (``ref_indices``).  Children are always 2^d (some
    possibly empty), ordered as itertools.product([le, gt], repeat=d).
    """

    def __init__(self, P, ndim, leaf_size=64, max_levels=64, parts=None):
        X = np.ascontiguousarray(P[:, :ndim], dtype=np.float64)
        N = X.shape[0]
        nch = 1 << ndim
        self.ndim = ndim
        self.nch = nch
        perm = np.arange(N, dtype=np.int64)
        start = [0]
        size = [N]
        level = [0]
        children = [None]
        lo_list = [X.min(0) if N else np.zeros(ndim)]
        hi_list = [X.max(0) if N else np.zeros(ndim)]
        frontier = np.array([0], dtype=np.int64) if N > leaf_size else np.zeros(0, np.int64)
        lev = 0
        if parts is not None:
            # the root's children are the given parts (a partition of the
            # facets, each in ascending order), split further as usual
            perm = np.concatenate([np.sort(np.asarray(I, np.int64)) for I in parts])
            ch, cs, nxt = [], 0, []
            for I in parts:
                n_c = int(np.size(I))
                cid = len(start)
                start.append(cs)
                size.append(n_c)
                level.append(1)
                children.append(None)
                if n_c:
                    seg_pts = X[perm[cs:cs + n_c]]
                    lo_list.append(seg_pts.min(0))
                    hi_list.append(seg_pts.max(0))
                    if n_c > leaf_size and not np.all(seg_pts.min(0) == seg_pts.max(0)):
                        nxt.append(cid)
                else:
                    lo_list.append(np.full(ndim, np.nan))
                    hi_list.append(np.full(ndim, np.nan))
                ch.append(cid)
                cs += n_c
            children[0] = ch
            frontier = np.array(nxt, dtype=np.int64)
            lev = 1
        while frontier.size and lev < max_levels:
            starts = np.array([start[f] for f in frontier], dtype=np.int64)
            sizes = np.array([size[f] for f in frontier], dtype=np.int64)
            idx = np.concatenate([perm[s:s + n] for s, n in zip(starts, sizes)])
            seg = np.repeat(np.arange(frontier.size), sizes)
            pts = X[idx]
            offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
            lo = np.minimum.reduceat(pts, offs, axis=0)
            hi = np.maximum.reduceat(pts, offs, axis=0)
            mid = (lo + hi) / 2
            code = np.zeros(idx.size, dtype=np.int64)
            for a in range(ndim):
                code |= (pts[:, a] > mid[seg, a]).astype(np.int64) << (ndim - 1 - a)
            order = np.lexsort((np.arange(idx.size), code, seg))
            new_idx = idx[order]
            counts = np.bincount(seg * nch + code, minlength=frontier.size * nch).reshape(-1, nch)
            new_frontier = []
            pos = 0
            for q, f in enumerate(frontier):
                s0 = starts[q]
                perm[s0:s0 + sizes[q]] = new_idx[pos:pos + sizes[q]]
                pos += sizes[q]
                ch = []
                cs = s0
                for c in range(nch):
                    cid = len(start)
                    n_c = int(counts[q, c])
                    start.append(int(cs))
                    size.append(n_c)
                    level.append(lev + 1)
                    children.append(None)
                    if n_c:
                        seg_pts = X[perm[cs:cs + n_c]]
                        lo_list.append(seg_pts.min(0))
                        hi_list.append(seg_pts.max(0))
                    else:
                        lo_list.append(np.full(ndim, np.nan))
                        hi_list.append(np.full(ndim, np.nan))
                    ch.append(cid)
                    if n_c > leaf_size and not np.all(seg_pts.min(0) == seg_pts.max(0)):
                        new_frontier.append(cid)
                    cs += n_c
                children[f] = ch
            frontier = np.array(new_frontier, dtype=np.int64)
            lev += 1
        self.perm = perm
        self.start = np.array(start, dtype=np.int64)
        self.size = np.array(size, dtype=np.int64)
        self.level = np.array(level, dtype=np.int64)
        self.children = children
        self.lo = np.array(lo_list)
        self.hi = np.array(hi_list)
        self.num_nodes = len(start)

    def indices(self, node):
        s = self.start[node]
        return self.perm[s:s + self.size[node]]

    def ref_indices(self, node):
        return np.sort(self.indices(node))


def _bbox3(P, tree):
    """3-D bounding boxes of every node (for admissibility)."""
    lo = np.full((tree.num_nodes, 3), np.nan)
    hi = np.full((tree.num_nodes, 3), np.nan)
    Pp = P[tree.perm]
    nz = np.where(tree.size > 0)[0]
    for node in nz:
        s, n = tree.start[node], tree.size[node]
        seg = Pp[s:s + n]
        lo[node] = seg.min(0)
        hi[node] = seg.max(0)
    return lo, hi


# ------------------------------------------------------------- builder --
LEAF_ZERO, LEAF_DENSE, LEAF_SPARSE, LEAF_LOWRANK, NODE = 0, 1, 2, 3, 4
# rank codes of fgb_aca_f64 besides k >= 0: not compressible (split the
# block), pool full, and "every entry known, the exact leaf is smaller"
ACA_FAILED, ACA_POOL_FULL, ACA_EXACT = -1, -2, -3


def _nbytes_csr(nnz, m, itemsize):
    # data + int32 indices + int32 indptr (scipy's index dtype for these sizes)
    return nnz * (itemsize + 4) + (m + 1) * 4


def _classify_exact(nnz, m, n, min_size, itemsize):
    """Kinds of exact leaves with nnz nonzeros in m x n: zero, dense when
    below min_size entries and smaller than CSR, else sparse (the
    reference's choice by bytes, compressed_form_factors.py:313-341)."""
    nnz = np.asarray(nnz, np.int64)
    mn = np.asarray(m, np.int64) * np.asarray(n, np.int64)
    dense = (mn < min_size) & (mn * itemsize < _nbytes_csr(nnz, np.asarray(m, np.int64), itemsize))
    return np.where(nnz == 0, LEAF_ZERO, np.where(dense, LEAF_DENSE, LEAF_SPARSE)).astype(np.int64)


def _admissible_blocks(lo3, hi3, r, c, eta):
    """min(diam_r, diam_c) <= eta dist(r, c) and dist > 0, per block (bounding
    boxes of the clusters)."""
    dr = np.linalg.norm(hi3[r] - lo3[r], axis=1)
    dc = np.linalg.norm(hi3[c] - lo3[c], axis=1)
    gap = np.maximum(0.0, np.maximum(lo3[r] - hi3[c], lo3[c] - hi3[r]))
    dist = np.linalg.norm(gap, axis=1)
    return (np.minimum(dr, dc) <= eta * dist) & (dist > 0)


def _plan_blocks(tree, lo3, hi3, *, tol, min_size, max_depth, force_max_depth, eta, run_aca):
    """The block tree of the compressed operator, level by level (the
    decisions of FormFactorBlockMatrix.make_block,
    compressed_form_factors.py:285-386, with ACA in place of the SVD):
    a block of an empty cluster is zero; at max_depth or between leaf
    clusters it is exact; below min_size entries exact; admissible blocks
    (tol > 0) go to ACA, and those ACA cannot compress are split (or exact
    where they cannot be); the rest is split into all child-cluster pairs.
    run_aca(r, c, pool_base) -> (ranks, offsets, pool part or None) for node
    id arrays r, c.  Block ids follow creation order: the root, its children,
    then per level the children of the blocks split in level order,
    followed by the children of the blocks ACA gave back.  Returns the block
    arrays, the exact leaves and the ACA pool parts."""
    nch = tree.nch
    nn = tree.num_nodes
    has_ch = np.array([ch is not None for ch in tree.children], bool)
    child_arr = np.full((nn, nch), -1, np.int64)
    for i in range(1, nn):
        ch = tree.children[i]
        if ch is not None:
            child_arr[i] = ch
    size = tree.size.astype(np.int64)
    parts = {k: [] for k in ("rows", "cols", "parent", "depth")}
    sets = {k: [] for k in ("kind", "child0", "rank", "pool_off")}
    count = [0]

    def add(r, c, p, d):
        k = r.size
        ids = np.arange(count[0], count[0] + k, dtype=np.int64)
        count[0] += k
        for key, v in (("rows", r), ("cols", c), ("parent", p), ("depth", d)):
            parts[key].append(np.asarray(v, np.int64))
        return ids

    def split(ids, r, c, d):
        """Children of blocks ids (in order): all pairs of child clusters."""
        k = ids.size
        cr, cc = child_arr[r], child_arr[c]
        R = np.broadcast_to(cr[:, :, None], (k, nch, nch)).reshape(-1)
        Cc = np.broadcast_to(cc[:, None, :], (k, nch, nch)).reshape(-1)
        new = add(R, Cc, np.repeat(ids, nch * nch), np.repeat(d + 1, nch * nch))
        sets["kind"].append((ids, np.full(k, NODE)))
        sets["child0"].append((ids, new[::nch * nch]))
        return new, R, Cc, np.repeat(d + 1, nch * nch)

    root = add(np.zeros(1), np.zeros(1), np.full(1, -1), np.zeros(1))
    sets["kind"].append((root, np.full(1, NODE)))
    ch_root = tree.children[0]
    if ch_root is None:
        lv = (add(np.zeros(1), np.zeros(1), np.zeros(1), np.ones(1)),
              np.zeros(1, np.int64), np.zeros(1, np.int64), np.ones(1, np.int64))
        root_bshape = (1, 1)
    else:
        cr = np.asarray(ch_root, np.int64)
        R, Cc = np.repeat(cr, cr.size), np.tile(cr, cr.size)
        one = np.ones(R.size, np.int64)
        lv = (add(R, Cc, np.zeros(R.size), one), R, Cc, one)
        root_bshape = (cr.size, cr.size)
    sets["child0"].append((root, lv[0][:1]))
    exact = []
    pool_parts = []
    aca_total = 0
    n_aca = n_failed = n_exact_pref = 0
    while lv[0].size:
        ids, r, c, d = lv
        m, n = size[r], size[c]
        zero = (m == 0) | (n == 0)
        at_max = (d >= max_depth) if max_depth is not None else np.zeros(ids.size, bool)
        can_split = has_ch[r] & has_ch[c] & ~at_max
        live = ~zero
        if force_max_depth and max_depth is not None:
            fsplit = live & can_split
        else:
            fsplit = np.zeros(ids.size, bool)
        live &= ~fsplit
        small = live & (m * n < min_size) & (not force_max_depth)
        live &= ~small
        cand = np.zeros(ids.size, bool)
        if tol > 0 and live.any():
            li = np.flatnonzero(live)
            cand[li] = _admissible_blocks(lo3, hi3, r[li], c[li], eta)
        live &= ~cand
        do_split = fsplit | (live & can_split)
        sets["kind"].append((ids[zero], np.full(int(zero.sum()), LEAF_ZERO)))
        exact.append(ids[small | (live & ~can_split)])
        nxt = []
        if do_split.any():
            nxt.append(split(ids[do_split], r[do_split], c[do_split], d[do_split]))
        if cand.any():
            ci = np.flatnonzero(cand)
            ranks, offs, pool = run_aca(r[ci], c[ci], aca_total)
            n_aca += ci.size
            if pool is not None:
                pool_parts.append(pool)
                aca_total += pool.numel()
            ok = ranks >= 0
            sets["kind"].append((ids[ci[ok]], np.full(int(ok.sum()), LEAF_LOWRANK)))
            sets["rank"].append((ids[ci[ok]], ranks[ok].astype(np.int64)))
            sets["pool_off"].append((ids[ci[ok]], offs[ok].astype(np.int64)))
            # ACA_EXACT: every entry was known and the exact leaf is smaller
            store = ci[ranks == ACA_EXACT]
            exact.append(ids[store])
            n_exact_pref += store.size
            bad = ci[(ranks < 0) & (ranks != ACA_EXACT)]
            n_failed += bad.size
            sp = bad[can_split[bad]]
            exact.append(ids[bad[~can_split[bad]]])
            if sp.size:
                nxt.append(split(ids[sp], r[sp], c[sp], d[sp]))
        if nxt:
            lv = tuple(np.concatenate([x[i] for x in nxt]) for i in range(4))
        else:
            lv = (np.zeros(0, np.int64),) * 4
    nb = count[0]
    out = {k: np.concatenate(v) for k, v in parts.items()}
    defaults = {"kind": -1, "child0": -1, "rank": 0, "pool_off": -1}
    for key, dflt in defaults.items():
        a = np.full(nb, dflt, np.int64)
        for ids, vals in sets[key]:
            a[ids] = vals
        out[key] = a
    out.update(exact=np.concatenate(exact) if exact else np.zeros(0, np.int64),
               aca_pool_parts=pool_parts, root_bshape=root_bshape, aca_blocks=n_aca,
               aca_failed=n_failed, aca_stored_exactly=n_exact_pref)
    return out


class fgb_op_desc(C.Structure):
    """ctypes mirror of struct fgb_op_desc (include/fluxgb.h)."""
    _fields_ = [
        ("g_c0", C.c_void_p), ("g_n", C.c_void_p), ("g_kz", C.c_void_p), ("g_ldv", C.c_void_p),
        ("g_voff", C.c_void_p), ("g_z0", C.c_void_p), ("a_grp", C.c_void_p),
        ("a_j0", C.c_void_p), ("a_j1", C.c_void_p), ("a_excl", C.c_void_p),
        ("num_items", C.c_longlong), ("t_p0", C.c_void_p), ("src", C.c_void_p),
        ("num_tiles", C.c_longlong), ("N", C.c_longlong), ("num_zrows", C.c_longlong),
        ("max_group_tiles", C.c_int), ("g_kzp", C.c_void_p), ("g_vtoff", C.c_void_p),
        ("a_woff", C.c_void_p), ("num_work", C.c_longlong), ("panel_rows", C.c_longlong),
        ("tile_rows", C.c_int), ("slice_rows", C.c_int), ("a_witem", C.c_void_p),
        ("tile_order", C.c_void_p),
    ]


TILE_ROWS = 64
ITEM_COLS = 2048
# panel rows per tile are padded to this multiple (the tensor-core phase-B
# kernel consumes 64 panel rows per pipeline stage)
PANEL_ALIGN = 64
# Z rows computed per CTA by the tensor-core phase A
TC_A_ROWS = 128


def _hilbert_index(x, y, order=16):
    """Index along the Hilbert curve of integer points (x, y) in
    [0, 2^order)^2 (the classic quadrant-by-quadrant construction)."""
    x = np.array(x, np.int64, copy=True)
    y = np.array(y, np.int64, copy=True)
    d = np.zeros_like(x)
    s = 1 << (order - 1)
    while s > 0:
        rx = ((x & s) > 0).astype(np.int64)
        ry = ((y & s) > 0).astype(np.int64)
        d += s * s * ((3 * rx) ^ ry)
        m = ry == 0
        flip = m & (rx == 1)
        x[flip] = s - 1 - x[flip]
        y[flip] = s - 1 - y[flip]
        t = x[m].copy()
        x[m] = y[m]
        y[m] = t
        s >>= 1
    return d


def _transpose_exact_csr(tcsr, ex_m, ex_n, chunk_nnz=200_000_000):
    """The exact leaves' device CSR (one tile per leaf, rows local to the
    leaf, columns local to it, visible-pair bitmask) of the transposed
    leaves: leaf q becomes an ex_n[q] x ex_m[q] tile with the same values.
    The entries of a leaf occupy the same range of the entry arrays before
    and after, so leaves are transposed in chunks of about chunk_nnz entries."""
    from .form_factors import TileCSR
    dev = tcsr.indptr.device
    nleaf = int(ex_m.size)
    ex_m = np.asarray(ex_m, np.int64)
    ex_n = np.asarray(ex_n, np.int64)
    ro = np.asarray(tcsr.row_off, np.int64)
    ro_t = np.zeros(nleaf + 1, np.int64)
    np.cumsum(ex_n, out=ro_t[1:])
    wpr_t = (ex_m + 31) // 32
    wo_t = np.zeros(nleaf + 1, np.int64)
    np.cumsum(ex_n * wpr_t, out=wo_t[1:])
    indptr = tcsr.indptr
    nnz = int(indptr[-1].item()) if indptr.numel() else 0
    indices_t = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    data_t = torch.empty(max(nnz, 1), dtype=tcsr.data.dtype, device=dev)
    counts_t = torch.zeros(int(ro_t[-1]) + 1, dtype=torch.int64, device=dev)
    bits64 = torch.zeros(max(int(wo_t[-1]), 1), dtype=torch.int64, device=dev)
    leaf_e0 = indptr[torch.as_tensor(ro, device=dev)].cpu().numpy()   # first entry of each leaf
    d = lambda a: torch.as_tensor(a, device=dev)
    ro_d, ro_t_d, wo_t_d, wpr_t_d = d(ro), d(ro_t), d(wo_t), d(wpr_t)
    q0 = 0
    while q0 < nleaf:
        q1 = int(np.searchsorted(leaf_e0, leaf_e0[q0] + chunk_nnz, side="right")) - 1
        q1 = min(max(q1, q0 + 1), nleaf)
        e0, e1 = int(leaf_e0[q0]), int(leaf_e0[q1])
        r0, r1 = int(ro[q0]), int(ro[q1])
        if e1 > e0:
            cnt = indptr[r0 + 1:r1 + 1] - indptr[r0:r1]
            row = torch.repeat_interleave(torch.arange(r0, r1, device=dev), cnt)
            leaf = torch.searchsorted(ro_d, row, right=True) - 1
            r = row - ro_d[leaf]
            del row
            c = tcsr.indices[e0:e1].to(torch.int64)
            g = ro_t_d[leaf] + c                    # transposed row
            key = g * int(ex_m[q0:q1].max() + 1) + r
            order = torch.argsort(key)
            del key
            indices_t[e0:e1] = r[order].to(torch.int32)
            data_t[e0:e1] = tcsr.data[e0:e1][order]
            counts_t.index_add_(0, g, torch.ones_like(g))
            word = wo_t_d[leaf] + c * wpr_t_d[leaf] + (r >> 5)
            bits64.index_add_(0, word, torch.ones_like(r) << (r & 31))
            del leaf, r, c, g, order, word
        q0 = q1
    indptr_t = torch.zeros(int(ro_t[-1]) + 1, dtype=torch.int64, device=dev)
    torch.cumsum(counts_t[:-1], 0, out=indptr_t[1:])
    bits = torch.where(bits64 >= 2**31, bits64 - 2**32, bits64).to(torch.int32)
    return TileCSR(indptr_t, indices_t[:nnz], data_t[:nnz], ro_t, tcsr.kept_pairs,
                   tcsr.near_edge_pairs, bits, wo_t)


class CompressedFormFactorMatrix(scipy.sparse.linalg.LinearOperator):
    """A compressed form factor (view factor) matrix
    (src/flux/compressed_form_factors.py:701-873)."""

    def __init__(self, shape_model, tol=1e-5, min_size=16384, max_depth=None,
                 force_max_depth=False, RootBlock=None, *, leaf_size=64, eta=1.0, rmax=64,
                 nsample=16384, exact_aca_max=262144, dtype=None, eps=None, aca_tol=None,
                 recompress=True, exact_zero_blocks=True, **kwargs):
        if tol < 0:
            raise RuntimeError('tol should be a nonnegative float')
        if max_depth is not None and not isinstance(max_depth, int):
            raise RuntimeError('invalid max_depth type: %s' % str(type(max_depth)))
        if isinstance(max_depth, int) and max_depth <= 0:
            raise RuntimeError('invalid max_depth value: %d' % max_depth)
        if force_max_depth and max_depth is None:
            raise RuntimeError('force_max_depth is True, but max_depth not specified')
        if rmax < 1 or rmax > 64:
            raise ValueError("rmax must be in [1, 64]")
        if RootBlock is None:
            RootBlock = FormFactorQuadtreeBlock
        self._parts = None
        self._ChildBlock = None
        if issubclass(RootBlock, FormFactorPartitionBlock):
            # compressed_form_factors.py:660-690: the rows and the columns
            # are split into the given parts first, then every (part, part)
            # block into the child block type
            parts = kwargs.get("parts")
            if parts is None:
                parts = [np.arange(shape_model.num_faces)]
            parts = [np.asarray(I, dtype=np.int64).ravel() for I in parts]
            union = np.unique(np.concatenate(parts)) if parts else np.zeros(0, np.int64)
            if union.size != sum(I.size for I in parts):
                raise Exception('parts must be disjoint')
            if union.size != shape_model.num_faces or (union.size and (
                    union[0] != 0 or union[-1] != shape_model.num_faces - 1)):
                raise ValueError("parts must cover every facet exactly once")
            self._parts = parts
            self._ChildBlock = kwargs.get("ChildBlock", FormFactorQuadtreeBlock)
        self.shape_model = shape_model
        self._tol = tol
        self._min_size = min_size
        self._max_depth = max_depth
        self._force_max_depth = force_max_depth
        self._RootBlock = RootBlock
        self._leaf_size = leaf_size
        self._eta = eta
        self._rmax = rmax
        self._nsample = nsample
        self._exact_aca_max = int(exact_aca_max)
        # ACA runs below the block tolerance and the FP64 truncation brings
        # every block to it (sigma_i / sigma_0 > tol kept, the reference's rule)
        self._recompress = bool(recompress)
        self._exact_zero_blocks = bool(exact_zero_blocks)
        self._aca_tol = float(aca_tol if aca_tol is not None else
                              (tol / 10 if recompress else tol))
        self._eps = config.DEFAULT_EPS if eps is None else eps
        self._store_dtype = np.dtype(shape_model.dtype if dtype is None else dtype)
        if self._store_dtype not in (np.float64, np.float32):
            raise ValueError("dtype must be float64 or float32")
        self._root_cache = None
        self.stats = {}
        self._build()

    @classmethod
    def from_shape_model(cls, shape_model, **kwargs):
        """Build from a shape model (alias of the constructor)."""
        return cls(shape_model, **kwargs)

    # -- LinearOperator plumbing ----------------------------------------
    @property
    def dtype(self):
        return self.shape_model.dtype

    @property
    def num_faces(self):
        return self.shape_model.num_faces

    @property
    def shape(self):
        return self.shape_model.num_faces, self.shape_model.num_faces

    @property
    def ndim(self):
        return 2

    @property
    def sparsity_threshold(self):
        return 2.0 / 3.0

    # -- build ------------------------------------------------------------
    def _build(self):
        import time
        t_start = time.perf_counter()
        sm = self.shape_model
        dev = sm._device
        P = np.asarray(sm.P, dtype=np.float64)
        split_cls = self._ChildBlock if self._parts is not None else self._RootBlock
        ndim = 3 if issubclass(split_cls, FormFactorOctreeBlock) else 2
        tree = ClusterTree(P, ndim, leaf_size=self._leaf_size, parts=self._parts)
        self._tree = tree
        lo3, hi3 = _bbox3(P, tree)
        N = P.shape[0]
        perm_d = torch.as_tensor(tree.perm, device=dev)
        self._perm_d = perm_d
        iperm = np.empty_like(tree.perm)
        iperm[tree.perm] = np.arange(N)
        self._iperm_d = torch.as_tensor(iperm, device=dev)

        tol = float(self._tol)
        t_aca = [0.0]

        def run_aca(r, c, base):
            t0 = time.perf_counter()
            out = self._run_aca(r, c, tree, perm_d, base)
            t_aca[0] += time.perf_counter() - t0
            return out

        plan = _plan_blocks(tree, lo3, hi3, tol=tol, min_size=self._min_size,
                            max_depth=self._max_depth, force_max_depth=self._force_max_depth,
                            eta=self._eta, run_aca=run_aca)
        self._rows, self._cols = plan["rows"], plan["cols"]
        self._parent, self._kind = plan["parent"], plan["kind"]
        self._child0, self._depth = plan["child0"], plan["depth"]
        self._rank = plan["rank"]
        self._root_bshape = plan["root_bshape"]
        exact = plan["exact"]
        if self._exact_zero_blocks:
            exact = np.concatenate([exact, self._visible_in_zero_blocks(perm_d)])
        t0 = time.perf_counter()
        self._assemble(exact, plan["aca_pool_parts"], plan["pool_off"])
        t_exact = time.perf_counter() - t0
        torch.cuda.synchronize()
        lrm = self._kind == LEAF_LOWRANK
        self.stats.update(build_s=time.perf_counter() - t_start, aca_s=t_aca[0], exact_s=t_exact,
                          aca_blocks=plan["aca_blocks"], aca_failed=plan["aca_failed"],
                          aca_stored_exactly=plan["aca_stored_exactly"],
                          lowrank_blocks=int(lrm.sum()),
                          exact_blocks=int(exact.size), num_blocks=int(self._rows.size),
                          lowrank_entries=int(np.sum(self._rank[lrm] *
                                                     (tree.size[self._rows[lrm]] +
                                                      tree.size[self._cols[lrm]]))))

    def _run_aca(self, r, c, tree, perm_d, pool_base):
        """ACA of the blocks with row clusters r and column clusters c (node
        id arrays); returns per block the rank (-1: not compressible under
        the cap), the pool offset and the new pool part."""
        sm = self.shape_model
        dev = sm._device
        if np.dtype(sm.dtype) != np.float64:
            raise NotImplementedError("low-rank compression needs a float64 shape model")
        P, Nn, A = sm.device_geometry()
        # largest blocks first
        sizes = tree.size[r] * tree.size[c]
        order = np.argsort(-sizes, kind="stable")
        rs, cs = r[order], c[order]
        r0 = tree.start[rs].astype(np.int32)
        m = tree.size[rs].astype(np.int32)
        c0 = tree.start[cs].astype(np.int32)
        n = tree.size[cs].astype(np.int32)
        nb = int(rs.size)
        mmax, nmax = int(m.max()), int(n.max())
        rmax = self._rmax
        per_cta = C.c_longlong()
        _lib.call("fgb_aca_scratch_floats", rmax, mmax, nmax, C.byref(per_cta))
        num_ctas = int(min(nb, 152 * 4))
        # cap the scratch at ~8 GB
        while num_ctas > 1 and num_ctas * per_cta.value * 4 > 8 * 2**30:
            num_ctas //= 2
        scratch = torch.empty(num_ctas * per_cta.value, dtype=torch.float32, device=dev)
        ex_max = self._exact_aca_max
        dscratch = torch.empty(max(num_ctas * ex_max, 1), dtype=torch.float32, device=dev)
        cap_k = np.minimum(rmax, np.maximum(1, (m.astype(np.int64) * n) // (2 * (m.astype(np.int64) + n))))
        capacity = int((cap_k * (m.astype(np.int64) + n)).sum())
        pool = torch.empty(max(capacity, 1), dtype=torch.float32, device=dev)
        used = torch.zeros(1, dtype=torch.int64, device=dev)
        rank_out = torch.empty(nb, dtype=torch.int32, device=dev)
        off_out = torch.empty(nb, dtype=torch.int64, device=dev)
        queue = torch.zeros(1, dtype=torch.int32, device=dev)
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
        t = lambda a: torch.as_tensor(a, device=dev)
        r0_d, m_d, c0_d, n_d = t(r0), t(m), t(c0), t(n)
        _lib.call("fgb_aca_f64", sm.bvh.handle, _lib.ptr(P), _lib.ptr(Nn), _lib.ptr(A),
                  _lib.ptr(perm_d), nb, _lib.ptr(r0_d), _lib.ptr(m_d), _lib.ptr(c0_d),
                  _lib.ptr(n_d), mmax, nmax, float(self._eps), sm.semantics, self._aca_tol,
                  rmax, self._nsample, ex_max, _lib.ptr(dscratch), _lib.ptr(scratch), num_ctas, _lib.ptr(pool), capacity,
                  _lib.ptr(used), _lib.ptr(rank_out), _lib.ptr(off_out), _lib.ptr(queue),
                  _lib.ptr(flags), _lib.stream_handle())
        fl = int(flags.item())
        if fl & _lib.FLAG_STACK_OVERFLOW:
            raise RuntimeError("BVH traversal stack overflow during compression")
        del scratch, dscratch
        nused = int(used.item())
        if self._recompress and nused and self._tol > 0:
            pool, nused = self._truncate(pool[:nused], rank_out, off_out, m_d, n_d)
        ranks_s = rank_out.cpu().numpy()
        offs_s = off_out.cpu().numpy()
        ranks = np.empty(nb, np.int64)
        offs = np.empty(nb, np.int64)
        ranks[order] = ranks_s
        offs[order] = np.where(offs_s >= 0, offs_s + pool_base, -1)
        return ranks, offs, (pool[:nused] if nused else None)

    def _visible_in_zero_blocks(self, perm_d, chunk_pairs=15_000_000_000):
        """Blocks that ACA found to be zero from its random samples but that
        hold visible pairs: every pair of those blocks is evaluated by the
        pair kernel (in chunks of about chunk_pairs pairs); the blocks with
        nonzeros become exact leaves (returned), the others stay zero.
        Occluded far-field blocks can hide a few pairs that see each other
        through a gap (thin slivers that no affordable random sample finds)."""
        import time
        t0 = time.perf_counter()
        tree = self._tree
        zb = np.flatnonzero((self._kind == LEAF_LOWRANK) & (self._rank == 0))
        r0 = tree.start[self._rows[zb]]
        m = tree.size[self._rows[zb]]
        c0 = tree.start[self._cols[zb]]
        n = tree.size[self._cols[zb]]
        pairs = m.astype(np.int64) * n
        found = []
        kept = 0
        lo = 0
        cum = np.cumsum(pairs)
        while lo < zb.size:
            base = cum[lo - 1] if lo else 0
            hi = int(np.searchsorted(cum, base + chunk_pairs, side="right"))
            hi = max(hi, lo + 1)
            sl = slice(lo, hi)
            tc = ff_tiles(self.shape_model, perm_d, perm_d, r0[sl], m[sl], c0[sl], n[sl],
                          self._eps)
            kept += tc.kept_pairs
            ro = torch.as_tensor(tc.row_off, device=perm_d.device)
            nnz = (tc.indptr[ro[1:]] - tc.indptr[ro[:-1]]).cpu().numpy()
            found.append(zb[sl][nnz > 0])
            del tc
            lo = hi
        out = np.concatenate(found) if found else np.zeros(0, np.int64)
        # these blocks are exact leaves now, no longer low-rank
        self._kind[out] = -1
        self._rank[out] = 0
        self.stats.update(zero_blocks_checked=int(zb.size), zero_blocks_with_pairs=int(out.size),
                          zero_block_pairs=int(pairs.sum()), zero_block_kept_pairs=int(kept),
                          zero_block_check_s=time.perf_counter() - t0)
        return out

    def _truncate(self, pool, rank, off, m_d, n_d):
        """FP64 rank truncation of the ACA factors of one batch of blocks
        (libfluxgb ``fgb_recompress_f32``): rank and off are updated in
        place; returns the new pool part and its length."""
        import time
        t0 = time.perf_counter()
        dev = pool.device
        nb = rank.numel()
        out = torch.empty(pool.numel(), dtype=torch.float32, device=dev)
        used = torch.zeros(1, dtype=torch.int64, device=dev)
        rank2 = torch.empty_like(rank)
        off2 = torch.empty_like(off)
        queue = torch.zeros(2, dtype=torch.int32, device=dev)
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("fgb_recompress_f32", _lib.ptr(pool), _lib.ptr(off), _lib.ptr(rank),
                  _lib.ptr(m_d), _lib.ptr(n_d), nb, float(self._tol), _lib.ptr(out), out.numel(),
                  _lib.ptr(used), _lib.ptr(rank2), _lib.ptr(off2), _lib.ptr(queue),
                  _lib.ptr(flags), _lib.stream_handle())
        fl = int(flags.item())
        if fl & (_lib.FLAG_NO_CONVERGE | _lib.FLAG_RANK_CAP | _lib.FLAG_INDEX_RANGE):
            raise RuntimeError(f"rank truncation of the ACA factors failed (flags {fl:#x})")
        ok = rank > 0
        st = self.stats
        st["aca_rank_sum"] = st.get("aca_rank_sum", 0) + int(rank[ok].sum().item())
        st["truncated_rank_sum"] = st.get("truncated_rank_sum", 0) + int(rank2[ok].sum().item())
        st["aca_factor_floats"] = st.get("aca_factor_floats", 0) + int(pool.numel())
        n = int(used.item())
        rank.copy_(rank2)
        off.copy_(off2)
        torch.cuda.synchronize()
        st["truncate_s"] = st.get("truncate_s", 0.0) + time.perf_counter() - t0
        return out[:n], n

    def _assemble(self, exact, aca_pool_parts, pool_off):
        """Exact leaves (sparse, from the pair kernel) and low-rank factors ->
        the flat panel layout of the device matvec."""
        sm = self.shape_model
        dev = sm._device
        tree = self._tree
        perm_d = self._perm_d
        sdt = self._store_dtype
        tdt = torch.float64 if sdt == np.float64 else torch.float32
        exact = np.sort(np.asarray(exact, dtype=np.int64))
        if exact.size:
            er = tree.start[self._rows[exact]]
            em = tree.size[self._rows[exact]]
            ec = tree.start[self._cols[exact]]
            exact = exact[np.lexsort((ec, em, er))]
        ex_r0 = tree.start[self._rows[exact]].astype(np.int64) if exact.size else np.zeros(0, np.int64)
        ex_m = tree.size[self._rows[exact]].astype(np.int64) if exact.size else np.zeros(0, np.int64)
        ex_c0 = tree.start[self._cols[exact]].astype(np.int64) if exact.size else np.zeros(0, np.int64)
        ex_n = tree.size[self._cols[exact]].astype(np.int64) if exact.size else np.zeros(0, np.int64)
        self._leaf_nnz = np.zeros(len(self._rows), np.int64)
        self._exact = exact
        # position of each exact leaf in the pair kernel's output (-1: none)
        self._exact_pos = np.full(len(self._rows), -1, np.int64)
        self._exact_pos[exact] = np.arange(exact.size)
        if exact.size:
            tcsr = ff_tiles(sm, perm_d, perm_d, ex_r0, ex_m, ex_c0, ex_n, self._eps,
                            keep_bits=True, out_dtype=tdt)
            self.stats["exact_nnz"] = int(tcsr.data.numel())
            self.stats["kept_pairs"] = tcsr.kept_pairs
            self.stats["near_edge_pairs"] = tcsr.near_edge_pairs
            ro = torch.as_tensor(tcsr.row_off, device=dev)
            nnz_leaf = (tcsr.indptr[ro[1:]] - tcsr.indptr[ro[:-1]]).cpu().numpy()
            self._leaf_nnz[exact] = nnz_leaf
            self._exact_csr = tcsr
        else:
            self._exact_csr = None
        # classify exact leaves as the reference would (zero / dense / CSR by bytes)
        isz = np.dtype(self.shape_model.dtype).itemsize
        self._kind[exact] = _classify_exact(self._leaf_nnz[exact], ex_m, ex_n,
                                            self._min_size, isz)
        aca = (torch.cat(aca_pool_parts) if aca_pool_parts else
               torch.zeros(1, dtype=torch.float32, device=dev))
        self._pool = aca.to(tdt)
        lr = np.where((self._kind == LEAF_LOWRANK) & (self._rank > 0))[0]
        self._layout(lr, pool_off, ex_r0, ex_m, ex_c0, ex_n)

    @staticmethod
    def _factor_offsets(off, k, m, n):
        """Pool offsets of U^T (k x m) and V^T (k x n) of low-rank blocks
        stored at `off` (U^T first)."""
        return off, off + k * m

    def _layout(self, lr, pool_off, ex_r0, ex_m, ex_c0, ex_n):
        """Panel layout consumed by libfluxgb's matvec kernels (matvec.cu)."""
        tree = self._tree
        dev = self.shape_model._device
        pool_off = np.asarray(pool_off, np.int64)
        N = self.num_faces
        stream = _lib.stream_handle()

        def d(a, dt):
            a = np.asarray(a, dtype=dt)
            return torch.as_tensor(a if a.size else np.zeros(1, dt), device=dev)

        # ---- low-rank blocks, grouped by column range (phase A)
        lr_r0 = tree.start[self._rows[lr]].astype(np.int64)
        lr_m = tree.size[self._rows[lr]].astype(np.int64)
        lr_c0 = tree.start[self._cols[lr]].astype(np.int64)
        lr_n = tree.size[self._cols[lr]].astype(np.int64)
        lr_k = self._rank[lr].astype(np.int64)
        lr_u, lr_v = self._factor_offsets(pool_off[lr], lr_k, lr_m, lr_n)
        order = np.lexsort((lr_n, lr_c0))
        lr, lr_r0, lr_m, lr_c0, lr_n, lr_k, lr_u, lr_v = (a[order] for a in
                                                         (lr, lr_r0, lr_m, lr_c0, lr_n, lr_k,
                                                          lr_u, lr_v))
        nlr = lr.size
        newg = np.ones(nlr, bool)
        if nlr:
            newg[1:] = (lr_c0[1:] != lr_c0[:-1]) | (lr_n[1:] != lr_n[:-1])
        gid = np.cumsum(newg) - 1
        ng = int(gid[-1]) + 1 if nlr else 0
        g_first = np.flatnonzero(newg)
        g_c0 = lr_c0[g_first]
        g_n = lr_n[g_first]
        g_kz = (np.bincount(gid, weights=lr_k, minlength=ng).astype(np.int64) if nlr
                else np.zeros(0, np.int64))
        g_ldv = (g_n + 7) // 8 * 8
        g_voff = np.zeros(ng + 1, np.int64)
        np.cumsum(g_kz * g_ldv, out=g_voff[1:])
        g_z0 = np.zeros(ng + 1, np.int64)
        np.cumsum(g_kz, out=g_z0[1:])
        lr_z = np.cumsum(lr_k) - lr_k          # groups are contiguous: first Z row
        self._num_zrows = int(g_z0[-1])
        vr_blk = np.repeat(np.arange(nlr), lr_k)
        vr_l = np.arange(lr_k.sum()) - np.repeat(np.cumsum(lr_k) - lr_k, lr_k)
        vr_src = lr_v[vr_blk] + vr_l * lr_n[vr_blk]
        vr_dst = g_voff[gid[vr_blk]] + (lr_z[vr_blk] - g_z0[gid[vr_blk]] + vr_l) * g_ldv[gid[vr_blk]]
        vr_n = lr_n[vr_blk]
        nchunk = (g_n + ITEM_COLS - 1) // ITEM_COLS
        a_grp = np.repeat(np.arange(ng), nchunk)
        ci = np.arange(nchunk.sum()) - np.repeat(np.cumsum(nchunk) - nchunk, nchunk)
        a_j0 = ci * ITEM_COLS
        a_j1 = np.minimum(g_n[a_grp], (ci + 1) * ITEM_COLS)
        a_ex = (nchunk[a_grp] == 1).astype(np.uint8)
        self._needs_zero_z = bool((a_ex == 0).any())
        max_gt = int(((g_kz + 63) // 64).max()) if ng else 1
        # tensor-core phase A: groups stored transposed (n x kz rounded up to
        # 64) and one work slice per (item, 64 rows of the group)
        # (kz rounded up to TC_A_ROWS: the tensor-core phase A computes
        # TC_A_ROWS rows of Z per CTA)
        g_kzp = (g_kz + TC_A_ROWS - 1) // TC_A_ROWS * TC_A_ROWS
        g_vtoff = np.zeros(ng + 1, np.int64)
        np.cumsum(g_n * g_kzp, out=g_vtoff[1:])
        # work slices of 64 rows (CUDA-core kernels) and of TC_A_ROWS rows
        # (tensor cores) per item
        a_wn = (g_kz[a_grp] + 63) // 64
        a_woff = np.zeros(a_grp.size + 1, np.int64)
        np.cumsum(a_wn, out=a_woff[1:])
        a_woff_tc = np.zeros(a_grp.size + 1, np.int64)
        np.cumsum(g_kzp[a_grp] // TC_A_ROWS, out=a_woff_tc[1:])
        # the tensor-core phase A with BF16 output takes one work item per
        # whole group (every CTA owns its output rows: no atomics, no FP32 Z)
        tg_woff = np.zeros(ng + 1, np.int64)
        np.cumsum(g_kzp // TC_A_ROWS, out=tg_woff[1:])
        # ... and, for the split products, 64-row slices (two CTAs per SM);
        # only slices that hold rows of the group
        tg_woff64 = np.zeros(ng + 1, np.int64)
        np.cumsum((g_kz + 63) // 64, out=tg_woff64[1:])
        # the item of every tensor-core work slice (no search per CTA)
        a_witem_tc = np.repeat(np.arange(a_grp.size), g_kzp[a_grp] // TC_A_ROWS)
        tg_witem = np.repeat(np.arange(ng), g_kzp // TC_A_ROWS)
        tg_witem64 = np.repeat(np.arange(ng), (g_kz + 63) // 64)
        tsl = g_kzp // 64
        tjb = (g_n + 63) // 64
        tcnt = tsl * tjb
        vt_g = np.repeat(np.arange(ng), tcnt)
        vt_i = np.arange(tcnt.sum()) - np.repeat(np.cumsum(tcnt) - tcnt, tcnt)
        vt_s = vt_i // np.repeat(tjb, tcnt)
        vt_j = vt_i % np.repeat(tjb, tcnt)
        ntiles = (N + TILE_ROWS - 1) // TILE_ROWS

        def tile_pairs(r0, m):
            t_first = r0 // TILE_ROWS
            cnt = (r0 + m - 1) // TILE_ROWS - t_first + 1
            pc = np.repeat(np.arange(r0.size), cnt)
            pt = np.repeat(t_first, cnt) + (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))
            return pc, pt

        # ---- phase B, low-rank part: (tile, LR block) pairs, k rows each
        lpc, lpt = tile_pairs(lr_r0, lr_m)
        o = np.argsort(lpt, kind="stable")
        lpc, lpt = lpc[o], lpt[o]
        lpk = lr_k[lpc]
        L_lr = np.bincount(lpt, weights=lpk, minlength=ntiles).astype(np.int64)
        # ---- phase B, near field: (tile, exact leaf) pairs, compacted columns
        nex = ex_r0.size
        tcsr = self._exact_csr
        self._nf = None
        if nex:
            npc, npt = tile_pairs(ex_r0, ex_m)
            o = np.argsort(npt, kind="stable")
            npc, npt = npc[o], npt[o]
            wpr = (ex_n + 31) // 32
            moff = np.zeros(npc.size + 1, np.int64)
            np.cumsum(wpr[npc], out=moff[1:])
            self._nf = dict(
                pair_q=d(npc, np.int32), pair_t0=d(npt * TILE_ROWS, np.int64),
                pair_moff=d(moff[:-1], np.int64), leaf_r0=d(ex_r0, np.int64),
                leaf_m=d(ex_m, np.int32), leaf_wpr=d(wpr, np.int32),
                leaf_word_off=d(tcsr.word_off[:-1], np.int64),
                leaf_row_off=d(tcsr.row_off[:-1], np.int64))
            mask = torch.empty(max(int(moff[-1]), 1), dtype=torch.int32, device=dev)
            cnt = torch.zeros(max(npc.size, 1), dtype=torch.int32, device=dev)
            nf = self._nf
            _lib.call("fgb_nf_pair_masks", _lib.ptr(nf["pair_q"]), _lib.ptr(nf["pair_t0"]),
                      _lib.ptr(nf["pair_moff"]), npc.size, int(moff[-1]), _lib.ptr(nf["leaf_r0"]),
                      _lib.ptr(nf["leaf_m"]), _lib.ptr(nf["leaf_wpr"]),
                      _lib.ptr(nf["leaf_word_off"]), _lib.ptr(nf["leaf_row_off"]),
                      _lib.ptr(tcsr.bits), _lib.ptr(mask), _lib.ptr(cnt), stream)
            npk = cnt[:npc.size].cpu().numpy().astype(np.int64)
            ndesc = int(npk.sum())
        else:
            npc = npt = npk = np.zeros(0, np.int64)
            ndesc = 0
            mask = None
        if ndesc:
            # one descriptor (pair, column) per set bit of the pair masks
            desc_off = np.zeros(npk.size + 1, np.int64)
            np.cumsum(npk, out=desc_off[1:])
            desc_pair = torch.empty(ndesc, dtype=torch.int32, device=dev)
            desc_col = torch.empty(ndesc, dtype=torch.int32, device=dev)
            nf = self._nf
            _lib.call("fgb_nf_enumerate", _lib.ptr(nf["pair_q"]), _lib.ptr(nf["pair_t0"]),
                      _lib.ptr(nf["pair_moff"]), npk.size, _lib.ptr(nf["leaf_wpr"]),
                      _lib.ptr(mask), _lib.ptr(d(desc_off[:-1], np.int64)), _lib.ptr(desc_pair),
                      _lib.ptr(desc_col), stream)
            # Exact leaves partition the matrix, so leaves that share a column
            # cluster cover disjoint rows: descriptors of one tile that gather
            # the same source column are merged into one panel row (each
            # fills only its own rows of it)
            dp = desc_pair.to(torch.int64)
            q_of = nf["pair_q"].to(torch.int64)[dp]
            tile_of = torch.as_tensor(npt, device=dev)[dp]
            c0_d = torch.as_tensor(ex_c0, device=dev)
            srcv = self._num_zrows + c0_d[q_of] + desc_col.to(torch.int64)
            del dp, q_of
            key = tile_of * (1 << 31) + srcv
            del tile_of, srcv
            skey, order = torch.sort(key)
            del key
            newrow = torch.ones(ndesc, dtype=torch.bool, device=dev)
            newrow[1:] = skey[1:] != skey[:-1]
            uid_sorted = torch.cumsum(newrow.to(torch.int64), 0) - 1
            ukeys = skey[newrow]
            del skey, newrow
            desc_uid = torch.empty(ndesc, dtype=torch.int64, device=dev)
            desc_uid[order] = uid_sorted
            del order, uid_sorted
            u_tile = ukeys >> 31
            u_src = ukeys & ((1 << 31) - 1)
            del ukeys
            L_nf = torch.bincount(u_tile, minlength=ntiles).cpu().numpy().astype(np.int64)
            self.stats["nearfield_descriptors"] = ndesc
        else:
            L_nf = np.zeros(ntiles, np.int64)
        L = L_lr + L_nf
        self._tile_L = L
        Lpad = (L + PANEL_ALIGN - 1) // PANEL_ALIGN * PANEL_ALIGN
        t_p0 = np.zeros(ntiles + 1, np.int64)
        np.cumsum(Lpad, out=t_p0[1:])
        total_rows = int(t_p0[-1])

        def offsets_within_tile(pt, pk):
            run = np.cumsum(pk) - pk
            first = np.ones(pt.size, bool)
            first[1:] = pt[1:] != pt[:-1]
            start = np.zeros(ntiles, np.int64)
            start[pt[first]] = run[first]
            return run - start[pt]

        lp0 = t_p0[lpt] + offsets_within_tile(lpt, lpk) if lpt.size else np.zeros(0, np.int64)
        # build-kernel pairs: LR pairs, plus one zero pair at every tile's
        # first near-field / padding row (rows past a pair's k are zeroed)
        tail_t = np.flatnonzero(Lpad > L_lr)
        tail_p0 = t_p0[tail_t] + L_lr[tail_t]
        all_p0 = np.concatenate([lp0, tail_p0])
        all_w = np.concatenate([lr_u[lpc], np.zeros(tail_t.size, np.int64)])
        all_m = np.concatenate([lr_m[lpc], np.ones(tail_t.size, np.int64)])
        all_shift = np.concatenate([lpt * TILE_ROWS - lr_r0[lpc], np.zeros(tail_t.size, np.int64)])
        all_k = np.concatenate([lpk, np.zeros(tail_t.size, np.int64)])
        oo = np.argsort(all_p0, kind="stable")
        all_p0, all_w, all_m, all_shift, all_k = (a[oo] for a in (all_p0, all_w, all_m, all_shift,
                                                                 all_k))
        # panel-row sources: LR rows -> Z rows (host), near-field rows -> X rows (device)
        src = np.zeros(total_rows, np.int64)
        rows_pair = np.repeat(np.arange(lpk.size), lpk)
        rows_l = np.arange(lpk.sum()) - np.repeat(np.cumsum(lpk) - lpk, lpk)
        src[lp0[rows_pair] + rows_l] = lr_z[lpc[rows_pair]] + rows_l
        src_d = d(src, np.int32)
        if ndesc:
            # merged rows: tile t's near-field rows start after its LR rows
            nf_start = torch.as_tensor(t_p0[:-1] + L_lr, device=dev)
            ufirst = torch.zeros(ntiles + 1, dtype=torch.int64, device=dev)
            ufirst[1:] = torch.cumsum(torch.as_tensor(L_nf, device=dev), 0)
            uidx = torch.arange(u_tile.numel(), device=dev)
            u_row = nf_start[u_tile] + (uidx - ufirst[u_tile])
            del uidx, ufirst, nf_start
            src_d[u_row] = u_src.to(torch.int32)
            desc_row = u_row[desc_uid]
            del u_row, u_src, u_tile, desc_uid
            self._nf.update(desc_pair=desc_pair, desc_col=desc_col, desc_row=desc_row)
            self._num_desc = ndesc
        else:
            self._num_desc = 0
        del mask
        if src.size and (self._num_zrows + N) >= 2**31:
            raise OverflowError("operator too large for 32-bit panel sources")
        self._dev = dict(
            g_c0=d(g_c0, np.int32), g_n=d(g_n, np.int32), g_kz=d(g_kz, np.int32),
            g_ldv=d(g_ldv, np.int32), g_voff=d(g_voff[:-1], np.int64), g_z0=d(g_z0[:-1], np.int64),
            a_grp=d(a_grp, np.int32), a_j0=d(a_j0, np.int32), a_j1=d(a_j1, np.int32),
            a_excl=d(a_ex, np.uint8), t_p0=d(t_p0, np.int64), src=src_d,
            g_kzp=d(g_kzp, np.int32), g_vtoff=d(g_vtoff[:-1], np.int64),
            a_woff=d(a_woff, np.int64), a_woff_tc=d(a_woff_tc, np.int64),
            a_witem_tc=d(a_witem_tc, np.int32))
        self._dev_tc = dict(
            a_grp=d(np.arange(ng), np.int32), a_j0=d(np.zeros(ng), np.int32),
            a_j1=d(g_n, np.int32), a_excl=d(np.ones(ng), np.uint8), a_woff=d(tg_woff, np.int64),
            a_woff64=d(tg_woff64, np.int64), a_witem=d(tg_witem, np.int32),
            a_witem64=d(tg_witem64, np.int32))
        self._build_dev = dict(
            vt_g=d(vt_g, np.int32), vt_s=d(vt_s, np.int32), vt_j=d(vt_j, np.int32),
            vr_src=d(vr_src, np.int64), vr_dst=d(vr_dst, np.int64), vr_n=d(vr_n, np.int32),
            p_p0=d(all_p0, np.int64), p_w=d(all_w, np.int64), p_m=d(all_m, np.int32),
            p_shift=d(all_shift, np.int64), p_k=d(all_k, np.int32))
        self._panel_rows = total_rows
        self._vpanel_size = int(g_voff[-1])
        self._vtpanel_size = int(g_vtoff[-1])
        self._num_vt_tiles = int(vt_g.size)
        self._num_vrows = int(vr_src.size)
        self._num_pairs = int(all_p0.size)
        self._desc = self._make_desc(int(a_grp.size), ntiles, max_gt, int(a_woff[-1]))
        self._desc_tc = self._make_desc_tc()
        self._desc_tc64 = self._make_desc_tc(64)
        self._desc_tc_items = self._make_desc_tc_items()
        self._lr_blocks = lr
        self._lr_u, self._lr_v = lr_u, lr_v
        self._panels = {}
        self._tc = {}
        self.stats.update(num_items=int(a_grp.size), num_tiles=ntiles, groups=ng,
                          panel_rows=total_rows, nearfield_rows=int(L_nf.sum()),
                          lowrank_rows=int(L_lr.sum()), max_group_tiles=max_gt,
                          pool_entries=int(self._pool.numel()), zrows=self._num_zrows,
                          operator_entries=int(total_rows * TILE_ROWS + g_voff[-1]))

    def _make_desc(self, num_items, ntiles, max_gt, num_work):
        desc = fgb_op_desc()
        for key in ("g_c0", "g_n", "g_kz", "g_ldv", "g_voff", "g_z0", "a_grp", "a_j0", "a_j1",
                    "a_excl", "t_p0", "src", "g_kzp", "g_vtoff", "a_woff"):
            setattr(desc, key, self._dev[key].data_ptr())
        desc.num_items = num_items
        desc.num_tiles = ntiles
        desc.N = self.num_faces
        desc.num_zrows = self._num_zrows
        desc.max_group_tiles = max_gt
        desc.num_work = num_work
        desc.panel_rows = int(self._panel_rows)
        desc.tile_rows = TILE_ROWS
        return desc

    def _make_desc_tc_items(self):
        """The descriptor with the column-split work items, in work slices of
        TC_A_ROWS rows (tensor-core phase A with FP32 output)."""
        desc = fgb_op_desc.from_buffer_copy(self._desc)
        desc.a_woff = self._dev["a_woff_tc"].data_ptr()
        desc.a_witem = self._dev["a_witem_tc"].data_ptr()
        desc.num_work = int(self._dev["a_woff_tc"][-1].item())
        return desc

    def _make_desc_tc(self, slice_rows=TC_A_ROWS):
        """The descriptor with one phase-A work item per whole group, in work
        slices of TC_A_ROWS rows, or of 64 rows (split products)."""
        desc = fgb_op_desc.from_buffer_copy(self._desc)
        woff = "a_woff" if slice_rows == TC_A_ROWS else "a_woff64"
        witem = "a_witem" if slice_rows == TC_A_ROWS else "a_witem64"
        for key in ("a_grp", "a_j0", "a_j1", "a_excl"):
            setattr(desc, key, self._dev_tc[key].data_ptr())
        desc.a_woff = self._dev_tc[woff].data_ptr()
        desc.a_witem = self._dev_tc[witem].data_ptr()
        desc.num_items = int(self._dev_tc["a_grp"].numel()) if self._num_zrows > 0 else 0
        desc.num_work = int(self._dev_tc[woff][-1].item())
        desc.slice_rows = slice_rows
        return desc

    # -- device products --------------------------------------------------
    def pool(self, precision):
        """The factor / dense pool (block storage) in 'fp64' or its own dtype."""
        if precision == "fp64" and self._pool.dtype != torch.float64:
            return self._pool.to(torch.float64)
        return self._pool

    _TDT = {"fp64": torch.float64, "fp32": torch.float32, "bf16": torch.bfloat16}

    def offload_pool(self, precisions=("fp32",)):
        """Build the panels of the given precisions, then move the block pool
        (needed only for other precisions and for block introspection) to
        host memory, freeing its device copy."""
        for p_ in precisions:
            self.panels(p_)
        self._pool = self._pool.cpu()
        tc = self._exact_csr
        if tc is not None:
            tc.data, tc.indptr, tc.bits, tc.indices = (tc.data.cpu(), tc.indptr.cpu(),
                                                       tc.bits.cpu(), tc.indices.cpu())
        torch.cuda.empty_cache()

    def panels(self, precision):
        """(phase-B panel, phase-A panel) in 'fp64', 'fp32' or 'bf16', built
        on first use from the pool."""
        got = self._panels.get(precision)
        if got is not None:
            return got
        tdt = self._TDT[precision]
        dev = self._perm_d.device
        if self._pool.device != dev:
            self._pool = self._pool.to(dev)
        pin = "f64" if self._pool.dtype == torch.float64 else "f32"
        pout = {"fp64": "f64", "fp32": "f32", "bf16": "bf16"}[precision]
        if pin == "f32" and pout == "f64":
            src = self._pool.to(torch.float64)
            pin = "f64"
        else:
            src = self._pool
        panel = torch.empty(max(self._panel_rows * TILE_ROWS, 8), dtype=tdt, device=dev)
        vpanel = torch.empty(max(self._vpanel_size, 8), dtype=tdt, device=dev)
        b = self._build_dev
        st = _lib.stream_handle()
        _lib.call(f"fgb_build_panel_{pin}_{pout}", _lib.ptr(src), self._panel_rows,
                  _lib.ptr(b["p_p0"]), _lib.ptr(b["p_w"]), _lib.ptr(b["p_m"]),
                  _lib.ptr(b["p_shift"]), _lib.ptr(b["p_k"]), self._num_pairs, _lib.ptr(panel), st)
        _lib.call(f"fgb_build_vpanel_{pin}_{pout}", _lib.ptr(src), self._num_vrows,
                  _lib.ptr(b["vr_src"]), _lib.ptr(b["vr_dst"]), _lib.ptr(b["vr_n"]),
                  _lib.ptr(vpanel), st)
        if self._num_desc:
            tc = self._exact_csr
            if tc.data.device != dev:
                tc.data, tc.indptr, tc.bits = tc.data.to(dev), tc.indptr.to(dev), tc.bits.to(dev)
            data = tc.data
            din = "f64" if data.dtype == torch.float64 else "f32"
            if din == "f32" and pout == "f64":
                data = data.to(torch.float64)
                din = "f64"
            nf = self._nf
            _lib.call(f"fgb_nf_fill_{din}_{pout}", _lib.ptr(nf["pair_q"]), _lib.ptr(nf["pair_t0"]),
                      int(nf["pair_q"].numel()), _lib.ptr(nf["leaf_r0"]), _lib.ptr(nf["leaf_m"]),
                      _lib.ptr(nf["leaf_wpr"]), _lib.ptr(nf["leaf_word_off"]),
                      _lib.ptr(nf["leaf_row_off"]), _lib.ptr(tc.bits), _lib.ptr(tc.indptr),
                      _lib.ptr(data), _lib.ptr(nf["desc_pair"]), _lib.ptr(nf["desc_col"]),
                      _lib.ptr(nf["desc_row"]), self._num_desc, _lib.ptr(panel), st)
        self._panels[precision] = (panel, vpanel)
        return panel, vpanel

    # keys of the device layout and caches that a transposed copy rebuilds
    _LAYOUT_KEYS = ("_dev", "_dev_tc", "_build_dev", "_nf", "_desc", "_desc_tc", "_desc_tc64",
                    "_desc_tc_items", "_desc128", "_dev128", "_desc256", "_dev256", "_panels",
                    "_tc", "_flags_d",
                    "_fgb_adjoint_ops", "_root_cache", "_host_tree_cache", "_transposed",
                    "_exact_csr", "_lr_blocks", "_lr_u", "_lr_v", "_tile_L")

    def transposed(self):
        """F^T as an operator of the same kind (cached): the same blocks with
        rows and columns exchanged, U and V exchanged in the low-rank blocks
        and the exact leaves' CSR transposed on the device, laid out in
        panels of its own.  Every product of F (K = 1 or K columns, FP32,
        FP64 arithmetic, BF16 tensor cores) is then available for F^T, with
        the same determinism (each output row tile written by one CTA)."""
        T = self.__dict__.get("_transposed")
        if T is not None:
            return T
        dev = self._perm_d.device
        if self._pool.device != dev:
            self._pool = self._pool.to(dev)
        tc = self._exact_csr
        if tc is not None and tc.indptr.device != dev:
            tc.data, tc.indptr, tc.bits, tc.indices = (tc.data.to(dev), tc.indptr.to(dev),
                                                       tc.bits.to(dev), tc.indices.to(dev))
        tree = self._tree
        exact = self._exact
        ex_r0 = tree.start[self._rows[exact]].astype(np.int64)
        ex_m = tree.size[self._rows[exact]].astype(np.int64)
        ex_c0 = tree.start[self._cols[exact]].astype(np.int64)
        ex_n = tree.size[self._cols[exact]].astype(np.int64)
        T = CompressedFormFactorMatrix.__new__(CompressedFormFactorMatrix)
        T.__dict__.update({k: v for k, v in self.__dict__.items() if k not in self._LAYOUT_KEYS})
        T._rows, T._cols = self._cols, self._rows
        T._root_cache = None
        T.stats = {}
        # a block's pool slot holds the original U^T (k x m) then V^T (k x n):
        # the transposed block's U^T is the original V^T, its V^T the original U^T
        T._factor_offsets = lambda off, k, m, n: (off + k * n, off)
        T._exact_csr = (_transpose_exact_csr(tc, ex_m, ex_n) if tc is not None else None)
        pool_off = np.full(len(self._rows), -1, np.int64)
        pool_off[self._lr_blocks] = self._lr_u
        lr = np.where((self._kind == LEAF_LOWRANK) & (self._rank > 0))[0]
        T._layout(lr, pool_off, ex_c0, ex_n, ex_r0, ex_m)
        T._is_transposed = True
        self._transposed = T
        return T

    def permute(self, x: torch.Tensor) -> torch.Tensor:
        """Facet order -> cluster order (rows)."""
        return x.index_select(0, self._perm_d)

    def unpermute(self, xp: torch.Tensor) -> torch.Tensor:
        return xp.index_select(0, self._iperm_d)

    def matvec_permuted(self, xp, precision="fp32", out=None, add=None, alpha=1.0, z=None):
        """y = F x (or add + alpha F x) in cluster order, K = 1.

        precision: 'fp32' (FP32 panels and arithmetic), 'fp64' (FP64 panels
        and arithmetic), 'fp32-fp64' (the FP32-stored operator applied in FP64
        arithmetic)."""
        if precision == "fp64":
            V = torch.float64
            fn = "fgb_matvec_f64"
            pp = "fp64"
        elif precision == "fp32-fp64":
            V = torch.float64
            fn = "fgb_matvec_f32_f64"
            pp = "fp32"
        else:
            V = torch.float32
            fn = "fgb_matvec_f32"
            pp = "fp32"
        xp = xp.to(V).contiguous()
        if out is None:
            out = torch.empty_like(xp)
        if z is None:
            z = torch.empty(max(self._num_zrows, 1), dtype=V, device=xp.device)
        panel, vpanel = self.panels(pp)
        _lib.call(fn, C.byref(self._desc), _lib.ptr(panel), _lib.ptr(vpanel), _lib.ptr(xp),
                  _lib.ptr(z), _lib.ptr(out), _lib.ptr(add), float(alpha),
                  int(self._needs_zero_z), _lib.stream_handle())
        return out

    def rmatvec_permuted(self, yp, precision=None):
        """F^T y in cluster order, K = 1, FP64 vectors and arithmetic.

        precision: 'fp64' (FP64 panels) or 'fp32-fp64' (the FP32-stored
        operator); default: the pool's own precision.  The product is the
        transposed operator's (``transposed()``), deterministic."""
        if precision is None:
            precision = "fp64" if self._pool.dtype == torch.float64 else "fp32-fp64"
        if precision not in ("fp64", "fp32-fp64"):
            raise ValueError(f"transpose products run in FP64 arithmetic, not {precision!r}")
        return self.transposed().matvec_permuted(yp.to(torch.float64).contiguous(), precision)

    def rmatmat_permuted(self, Yp, precision=None):
        """F^T Y in cluster order for Y (N, K) (the transposed operator's
        products: 'fp32', 'bf16', 'fp32-fp64' all columns at once, 'fp64'
        column by column; default: FP64 arithmetic)."""
        if precision is None:
            precision = "fp64" if self._pool.dtype == torch.float64 else "fp32-fp64"
        return self.transposed().matmat_permuted(Yp.contiguous(), precision)

    def matmat_permuted(self, Xp, precision="fp32", out=None, add=None, alpha=1.0, Z=None):
        """Y = F X for K right-hand sides in cluster order (X: N x K)."""
        K = Xp.shape[1]
        if precision == "fp64":
            # FP64: one column at a time (reference-precision path)
            cols = [self.matvec_permuted(Xp[:, c].contiguous(), "fp64",
                                         add=None if add is None else add[:, c].contiguous(),
                                         alpha=alpha) for c in range(K)]
            res = torch.stack(cols, 1)
            if out is not None:
                out.copy_(res)
                return out
            return res
        if precision == "fp32":
            Xp = Xp.to(torch.float32).contiguous()
            if out is None:
                out = torch.empty_like(Xp)
            if Z is None:
                Z = torch.empty((max(self._num_zrows, 1), K), dtype=torch.float32, device=Xp.device)
            panel, vpanel = self.panels("fp32")
            _lib.call("fgb_matmat_f32", C.byref(self._desc), _lib.ptr(panel), _lib.ptr(vpanel),
                      _lib.ptr(Xp), _lib.ptr(Z), _lib.ptr(out), K, _lib.ptr(add), float(alpha),
                      int(self._needs_zero_z), 3, _lib.stream_handle())
            return out
        if precision == "fp32-fp64":
            # the FP32-stored operator in FP64 arithmetic, all K columns at once
            Xp = Xp.to(torch.float64).contiguous()
            if out is None:
                out = torch.empty_like(Xp)
            if Z is None:
                Z = torch.empty((max(self._num_zrows, 1), K), dtype=torch.float64,
                                device=Xp.device)
            panel, vpanel = self.panels("fp32")
            addc = None if add is None else add.to(torch.float64).contiguous()
            _lib.call("fgb_matmat_f32_f64", C.byref(self._desc), _lib.ptr(panel), _lib.ptr(vpanel),
                      _lib.ptr(Xp), _lib.ptr(Z), _lib.ptr(out), K, _lib.ptr(addc), float(alpha),
                      int(self._needs_zero_z), _lib.stream_handle())
            return out
        if precision == "bf16":
            return self._matmat_bf16(Xp, out=out, add=add, alpha=alpha, Z=Z)
        raise ValueError(precision)

    def _matmat_bf16(self, Xp, out=None, add=None, alpha=1.0, Z=None, engine="tc"):
        K = Xp.shape[1]
        S, Zb, Xb = self.stacked_sources(K, Xp.device)
        Xb.copy_(Xp)
        if out is None:
            out = torch.empty(Xp.shape, dtype=torch.float32, device=Xp.device)
        if Z is None:
            Z = torch.empty((max(self._num_zrows, 1), K), dtype=torch.float32, device=Xp.device)
        self.bf16_product(Xb, Z, Zb, out, add, alpha, engine)
        return out

    def stacked_sources(self, K, device, buf=None):
        """A BF16 (num_zrows + N) x K tensor S with its two views Z = S[:num_zrows]
        and X = S[num_zrows:]: the phase-B sources stacked as the TMA gather
        kernel wants them (any Z / X pair works, stacked ones are faster)."""
        zr = self._num_zrows
        if buf is None or tuple(buf.shape) != (zr + self.num_faces, K):
            buf = torch.empty((zr + self.num_faces, K), dtype=torch.bfloat16, device=device)
        return buf, buf[:zr], buf[zr:]

    def _build_tc128(self, panel32, split=False):
        """The 128-row phase-B layout for the BF16 tensor-core products: the
        64-row panel's rows of tiles 2t and 2t + 1 that gather the same
        source become one 128-weight row of tile t (each source appears at
        most once per 64-row tile, so the halves never collide).  Returns
        (hi, lo): BF16 weights, and with split their low parts (else None)."""
        return self._build_tc_wide(panel32, 128, split)

    def _build_tc_wide(self, panel32, width, split=False):
        """Phase-B layout with tiles of `width` rows (128 or 256) for the
        BF16 tensor-core products: the 64-row panel's rows of the width / 64
        tiles that form one wide tile and gather the same source become one
        row of `width` weights (64-row tile t fills part t mod (width / 64)).
        Sets the layout's descriptor (_desc128 / _desc256) and returns (hi,
        lo) as _build_tc128 does; lo only for width 128."""
        assert width in (128, 256) and not (split and width != 128)
        parts = width // 64
        shift = parts.bit_length() - 1
        dev = panel32.device
        t_p0 = self._dev["t_p0"]
        ntiles = int(t_p0.numel() - 1)
        P = int(self._panel_rows)
        counts = t_p0[1:] - t_p0[:-1]
        tile = torch.repeat_interleave(torch.arange(ntiles, device=dev), counts)
        pos = torch.arange(P, device=dev) - t_p0[:-1][tile]
        Lt = torch.as_tensor(self._tile_L, device=dev)
        vidx = torch.nonzero(pos < Lt[tile]).squeeze(1)     # rows that are not padding
        del pos
        vtile = tile[vidx]
        half = (tile & (parts - 1)).to(torch.uint8)
        del tile
        vkey = (vtile >> shift) * (1 << 31) + self._dev["src"].to(torch.int64)[vidx]
        del vtile
        skey, order = torch.sort(vkey)
        del vkey
        newflag = torch.ones(skey.numel(), dtype=torch.bool, device=dev)
        newflag[1:] = skey[1:] != skey[:-1]
        uid_sorted = torch.cumsum(newflag.to(torch.int64), 0) - 1
        ukeys = skey[newflag]
        del skey, newflag
        u_tile = ukeys >> 31
        u_src = (ukeys & ((1 << 31) - 1)).to(torch.int32)
        del ukeys
        nt2 = (self.num_faces + width - 1) // width
        L2 = torch.bincount(u_tile, minlength=nt2)
        t2 = torch.zeros(nt2 + 1, dtype=torch.int64, device=dev)
        t2[1:] = torch.cumsum((L2 + PANEL_ALIGN - 1) // PANEL_ALIGN * PANEL_ALIGN, 0)
        ufirst = torch.zeros(nt2 + 1, dtype=torch.int64, device=dev)
        ufirst[1:] = torch.cumsum(L2, 0)
        u_row = t2[u_tile] + torch.arange(u_tile.numel(), device=dev) - ufirst[u_tile]
        del ufirst, u_tile
        new_row = torch.full((P,), -1, dtype=torch.int64, device=dev)
        new_row[vidx[order]] = u_row[uid_sorted]
        del vidx, order, uid_sorted
        total2 = int(t2[-1].item())
        src2 = torch.zeros(max(total2, 1), dtype=torch.int32, device=dev)
        src2[u_row] = u_src
        del u_row, u_src
        w128 = torch.zeros(max(total2, 1) * width, dtype=torch.bfloat16, device=dev)
        lo128 = None
        if width != 128:
            _lib.call("fgb_retile_panel_bf16_n", _lib.ptr(panel32), P, _lib.ptr(new_row),
                      _lib.ptr(half), width, _lib.ptr(w128), _lib.stream_handle())
        elif split:
            lo128 = torch.zeros_like(w128)
            _lib.call("fgb_retile_panel_split_bf16", _lib.ptr(panel32), P, _lib.ptr(new_row),
                      _lib.ptr(half), _lib.ptr(w128), _lib.ptr(lo128), _lib.stream_handle())
        else:
            _lib.call("fgb_retile_panel_bf16", _lib.ptr(panel32), P, _lib.ptr(new_row),
                      _lib.ptr(half), _lib.ptr(w128), _lib.stream_handle())
        del new_row, half
        desc = fgb_op_desc.from_buffer_copy(self._desc)
        desc.t_p0 = t2.data_ptr()
        desc.src = src2.data_ptr()
        desc.num_tiles = nt2
        desc.panel_rows = total2
        desc.tile_rows = width
        order = self._hilbert_tile_order(width, nt2, dev)
        desc.tile_order = order.data_ptr()
        setattr(self, f"_dev{width}", dict(t_p0=t2, src=src2, tile_order=order))
        setattr(self, f"_desc{width}", desc)
        self.stats[f"panel_rows_{width}"] = total2
        return w128, lo128

    def _hilbert_tile_order(self, width, ntiles, dev):
        """The order in which the tensor-core phase B takes its tiles of
        `width` rows: along a Hilbert curve through the tiles' centroids,
        projected on the two axes of largest extent (neighbouring tiles
        gather many of the same source rows; at 522k facets this ran 1 %
        faster than cluster order, a random order 12 % slower)."""
        N = self.num_faces
        P = np.asarray(self.shape_model.P, np.float64)[self._tree.perm]
        tile = np.arange(N) // width
        cnt = np.maximum(np.bincount(tile, minlength=ntiles), 1)
        cent = np.stack([np.bincount(tile, weights=P[:, a], minlength=ntiles) / cnt
                         for a in range(3)], 1)
        ext = cent.max(0) - cent.min(0)
        ax = np.argsort(-ext, kind="stable")[:2]
        q = ((cent[:, ax] - cent[:, ax].min(0)) / np.maximum(ext[ax], 1e-300) * 65535.0)
        key = _hilbert_index(q[:, 0].astype(np.int64), q[:, 1].astype(np.int64))
        order = np.argsort(key, kind="stable").astype(np.int32)
        return torch.as_tensor(order, device=dev)

    def tc_operands256(self):
        """The 256-row phase-B panel ('w256', BF16) of the plain product's
        widest layout, in the same dict as tc_operands; built on request."""
        tc = self.tc_operands()
        if "w256" not in tc or self.__dict__.get("_desc256") is None:
            panel, _ = self.panels("fp32")
            tc["w256"], _ = self._build_tc_wide(panel, 256)
        return tc

    def tc_operands(self, split=False):
        """BF16 operands of the tensor-core products, built once from the
        FP32 panels: 'w128' (phase-B panel with 128-row tiles, for the plain
        product) and 'vt_hi' (transposed phase-A panel) and, for split
        products, the 64-row phase-B panel 'w_hi' / 'w_lo' and 'vt_lo'
        (hi = bf16(v), lo = bf16(v - hi))."""
        tc = self.__dict__.setdefault("_tc", {})
        need = ("w128", "vt_hi") + (("w_hi", "w_lo", "vt_lo") if split else ())
        if all(k in tc for k in need):
            return tc
        panel, vpanel = self.panels("fp32")
        dev = panel.device
        st = _lib.stream_handle()
        if "w128" not in tc:
            tc["w128"], _ = self._build_tc128(panel)
        if "vt_hi" not in tc or (split and "vt_lo" not in tc):
            nvt = max(self._vtpanel_size, 8)
            vt_hi = tc.get("vt_hi")
            if vt_hi is None:
                vt_hi = torch.zeros(nvt, dtype=torch.bfloat16, device=dev)
            vt_lo = torch.zeros(nvt, dtype=torch.bfloat16, device=dev) if split else None
            b = self._build_dev
            _lib.call("fgb_vpanel_transpose_bf16", C.byref(self._desc), _lib.ptr(vpanel),
                      _lib.ptr(b["vt_g"]), _lib.ptr(b["vt_s"]), _lib.ptr(b["vt_j"]),
                      self._num_vt_tiles, _lib.ptr(vt_hi), _lib.ptr(vt_lo), st)
            tc["vt_hi"] = vt_hi
            if split:
                tc["vt_lo"] = vt_lo
        if split:
            self.tc_operands64(split=True)
        return tc

    def tc_operands64(self, split=False):
        """The 64-row phase-B panel in BF16, 'w_hi' (and its low part 'w_lo'
        with split), in the same dict as tc_operands: the operand of the
        split products and of the 64-row kernels (the TMA gather variant,
        comparisons)."""
        tc = self.__dict__.setdefault("_tc", {})
        if "w_hi" in tc and (not split or "w_lo" in tc):
            return tc
        panel, _ = self.panels("fp32")
        w_hi = tc.get("w_hi")
        if w_hi is None:
            w_hi = torch.empty(panel.numel(), dtype=torch.bfloat16, device=panel.device)
        w_lo = torch.empty_like(w_hi) if split else None
        _lib.call("fgb_split_bf16", _lib.ptr(panel), _lib.ptr(w_hi), _lib.ptr(w_lo),
                  panel.numel(), _lib.stream_handle())
        tc["w_hi"] = w_hi
        if split:
            tc["w_lo"] = w_lo
        return tc

    def tc_split128(self):
        """hi and lo parts of the 128-row phase-B panel for split products
        on 128-row tiles (8 warps and two CTAs per SM, the drained windows
        summed in plain FP32).  At 522k facets and 1,024 columns the split
        phase B took 71 ms on them against 106 ms on the 64-row tiles, with
        the same product error; autotune_products chooses between them."""
        panel, _ = self.panels("fp32")
        return self._build_tc128(panel, split=True)

    def bf16_product(self, Xb, Z, Zb, Y, add=None, alpha=1.0, engine="tc"):
        """Y = add + alpha F X with BF16 operands (X: N x K bf16, K % 8 == 0)
        and FP32 accumulation, in cluster order; Z (FP32) and Zb (BF16) are
        num_zrows x K scratch.  engine 'tc': both phases on the tcgen05
        tensor cores (TMEM accumulators); 'mma': mma.sync kernels."""
        K = Xb.shape[1]
        st = _lib.stream_handle()
        if engine == "mma":
            panel, vpanel = self.panels("bf16")
            _lib.call("fgb_matmat_bf16", C.byref(self._desc), _lib.ptr(panel), _lib.ptr(vpanel),
                      _lib.ptr(Xb), _lib.ptr(Z), _lib.ptr(Zb), _lib.ptr(Y), K, _lib.ptr(add),
                      float(alpha), int(self._needs_zero_z), 3, st)
            return Y
        tc = self.tc_operands()
        flags = _lib.ptr(self.device_flags())
        if self._num_zrows > 0:
            # phase A writes Z directly in BF16 (Z, the FP32 scratch, is unused)
            _lib.call("fgb_tc_phase_a_bf16", C.byref(self._desc_tc), _lib.ptr(tc["vt_hi"]), None,
                      _lib.ptr(Xb), None, _lib.ptr(Zb), None, K, flags, st)
        plain = self.product_plan()["plain"]
        if plain == "b64":
            desc, w = self._desc, self.tc_operands64()["w_hi"]
        elif plain == "b256":
            w = self.tc_operands256()["w256"]
            desc = self._desc256
        else:
            desc, w = self._desc128, tc["w128"]
        _lib.call("fgb_tc_phase_b", C.byref(desc), _lib.ptr(w), None,
                  _lib.ptr(Xb), None, _lib.ptr(Zb), None, _lib.ptr(Y), K, _lib.ptr(add),
                  float(alpha), flags, st)
        return Y

    def split_product(self, X, Y, add=None, alpha=1.0, work=None):
        """Y = add + alpha F X for FP32 X (N x K, K % 8 == 0) on the tensor
        cores with split-BF16 operands (hi.hi + lo.hi + hi.lo; the tensor
        core's FP32 accumulators are drained every 256 reduction rows into
        register sums, compensated on 64-row tiles).  Each product term is
        exact and the
        split operands carry ~17 significant bits, so the result behaves
        like FP32 arithmetic with 7 fewer bits.  work: optional dict of
        scratch tensors (reused)."""
        N, K = X.shape
        dev = X.device
        st = _lib.stream_handle()
        zr = max(self._num_zrows, 1)
        w = work if work is not None else {}

        def buf(name, shape, dt):
            t = w.get(name)
            if t is None or tuple(t.shape) != tuple(shape) or t.dtype != dt:
                t = w[name] = torch.empty(shape, dtype=dt, device=dev)
            return t
        # stacked [Z; X] sources, hi and lo parts (TMA gathers)
        nz = self._num_zrows
        sh = buf("s_hi", (nz + N, K), torch.bfloat16)
        sl = buf("s_lo", (nz + N, K), torch.bfloat16)
        zh, xh = sh[:nz], sh[nz:]
        zl, xl = sl[:nz], sl[nz:]
        plan = self.product_plan()["split"]
        # the operands this plan reads (the 64-row parts only for b64 tiles)
        tc = self.tc_operands()
        if "vt_lo" not in tc or (not plan.endswith("b128") and "w_lo" not in tc):
            tc = self.tc_operands(split=True)
        flags = _lib.ptr(self.device_flags())
        _lib.call("fgb_split_bf16", _lib.ptr(X), _lib.ptr(xh), _lib.ptr(xl), N * K, st)
        if self._num_zrows > 0:
            # phase A writes the hi / lo BF16 parts of Z directly: 64-row work
            # slices or 128-row ones (two CTAs per SM either way)
            dA = self._desc_tc if plan.startswith("a128") else self._desc_tc64
            _lib.call("fgb_tc_phase_a_bf16", C.byref(dA), _lib.ptr(tc["vt_hi"]),
                      _lib.ptr(tc["vt_lo"]), _lib.ptr(xh), _lib.ptr(xl), _lib.ptr(zh),
                      _lib.ptr(zl), K, flags, st)
        if plan.endswith("b128"):
            # 128-row tiles: the hi part is the plain product's panel
            dB, wh, wl = self._desc128, tc["w128"], self._split128_lo()
        else:
            dB, wh, wl = self._desc, tc["w_hi"], tc["w_lo"]
        _lib.call("fgb_tc_phase_b", C.byref(dB), _lib.ptr(wh), _lib.ptr(wl), _lib.ptr(xh),
                  _lib.ptr(xl), _lib.ptr(zh), _lib.ptr(zl), _lib.ptr(Y), K, _lib.ptr(add),
                  float(alpha), flags, st)
        return Y

    # -- product plans (autotuned) ------------------------------------------
    # plain BF16 product: phase-B tiles of 128 rows (merged tile pairs), 64
    # or 256 (merged tile quadruples)
    PLAIN_PLANS = ("b128", "b64", "b256")
    # split product: phase-A work slices of 64 / 128 rows, phase-B tiles of 64 / 128
    SPLIT_PLANS = ("a64-b64", "a128-b64", "a64-b128", "a128-b128")

    def product_plan(self):
        """Kernel layouts used by bf16_product and split_product: the
        defaults, or what autotune_products measured fastest."""
        return self.__dict__.setdefault("_plan", {"plain": "b128", "split": "a64-b64"})

    def _split128_lo(self):
        tc = self.tc_operands()
        if "w128_lo" not in tc:
            panel, _ = self.panels("fp32")
            _, tc["w128_lo"] = self._build_tc128(panel, split=True)
        return tc["w128_lo"]

    def autotune_products(self, K, reps=3, plans=None):
        """Time every kernel layout of the BF16 and split-BF16 products on this
        operator at K right-hand-side columns (CUDA events, after one warm-up
        product each) and keep the fastest in product_plan().  A layout whose
        extra operand does not fit in free device memory is skipped.  Returns
        {'plain': {plan: ms}, 'split': {plan: ms}, 'chosen': plan dict}; also
        kept in stats['autotune'].  The candidates compute the same product
        (up to the order of FP32 sums)."""
        if K < 8 or K % 8:
            raise ValueError("K must be a positive multiple of 8")
        dev = self._perm_d.device
        N = self.num_faces
        plans = plans or {"plain": self.PLAIN_PLANS, "split": self.SPLIT_PLANS}
        tc = self.tc_operands(split=True)
        g = torch.Generator(device=dev).manual_seed(0)
        X = torch.rand((N, K), generator=g, device=dev, dtype=torch.float32)
        Y = torch.empty_like(X)
        Sb, Zb, Xb = self.stacked_sources(K, dev)
        Xb.copy_(X)
        work = {"s_hi": Sb}     # as the solver does: the split sources reuse Sb
        plan = self.product_plan()
        old = dict(plan)
        stream = torch.cuda.current_stream()

        def timed(fn):
            fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            return a.elapsed_time(b) / reps

        table = {"plain": {}, "split": {}}
        for p_ in plans["plain"]:
            if p_ == "b256" and "w256" not in tc:
                # at most as many rows as the 128-row panel, twice as wide
                need = 2 * tc["w128"].numel() * 2 + (1 << 33)
                if torch.cuda.mem_get_info(dev)[0] < need:
                    table["plain"][p_] = None
                    continue
            plan["plain"] = p_
            table["plain"][p_] = timed(lambda: self.bf16_product(Xb, None, Zb, Y))
        for p_ in plans["split"]:
            if p_.endswith("b128") and "w128_lo" not in tc:
                # the 128-row split layout is built as hi and lo parts
                need = 2 * tc["w128"].numel() * 2 + (1 << 33)
                if torch.cuda.mem_get_info(dev)[0] < need:
                    table["split"][p_] = None   # does not fit beside the other operands
                    continue
            plan["split"] = p_
            table["split"][p_] = timed(lambda: self.split_product(X, Y, work=work))
        self.check_device_flags()
        best = {k: min((t, p_) for p_, t in v.items() if t is not None)[1]
                for k, v in table.items() if any(t is not None for t in v.values())}
        plan.update(old)
        plan.update(best)
        # give back the memory of the layouts not chosen (built again on
        # request)
        if not plan["split"].endswith("b128"):
            tc.pop("w128_lo", None)
        elif plan["plain"] != "b64":
            tc.pop("w_hi", None)         # the 64-row BF16 parts (2 x 20 GB at 522k)
            tc.pop("w_lo", None)
        if plan["plain"] != "b256":
            tc.pop("w256", None)
        del X, Y, Sb, Zb, Xb, work
        torch.cuda.empty_cache()
        table["chosen"] = dict(plan)
        self.stats["autotune"] = table
        return table

    def device_flags(self):
        """Device status word (FGB_FLAG_*) of the operator's kernels."""
        f = getattr(self, "_flags_d", None)
        if f is None or f.device != self._perm_d.device:
            f = self._flags_d = torch.zeros(1, dtype=torch.int32, device=self._perm_d.device)
        return f

    def check_device_flags(self):
        """Raise if a kernel of this operator reported a failure (synchronises)."""
        f = int(self.device_flags().item())
        if f:
            self._flags_d.zero_()
            if f & _lib.FLAG_DEVICE_TIMEOUT:
                raise RuntimeError("tensor-core product: a bounded device wait ran out")
            raise RuntimeError(f"operator kernel reported flags 0x{f:x}")

    def _default_precision(self):
        return "fp64" if self._pool.dtype == torch.float64 else "fp32"

    def _matmat(self, x):
        """Product with host or device input (shape (N,) or (N, K))."""
        on_dev = isinstance(x, torch.Tensor)
        dev = self.shape_model._device
        prec = self._default_precision()
        V = torch.float64 if prec == "fp64" else torch.float32
        xt = x if on_dev else torch.as_tensor(np.asarray(x), device=dev)
        if xt.dtype not in (torch.float32, torch.float64):
            xt = xt.to(V)
        orig_dtype = xt.dtype
        vec = xt.ndim == 1
        xp = self.permute(xt.to(V))
        if vec:
            yp = self.matvec_permuted(xp, prec)
        else:
            yp = self.matmat_permuted(xp, prec)
        y = self.unpermute(yp)
        if on_dev:
            return y.to(orig_dtype)
        return y.cpu().numpy().astype(self.dtype, copy=False)

    def _matvec(self, x):
        return self._matmat(x)

    def _rmatvec(self, x):
        """F^T x (host or device input, shape (N,) or (N, K)) in FP64
        arithmetic: what ``x @ F`` gives for the reference's sparse and dense
        form-factor matrices (CompressedKernelMatrix._rmatvec,
        compressed_form_factors.py:904-913)."""
        on_dev = isinstance(x, torch.Tensor)
        xt = x if on_dev else torch.as_tensor(np.asarray(x), device=self.shape_model._device)
        orig_dtype = xt.dtype
        xp = self.permute(xt.to(torch.float64))
        yp = self.rmatvec_permuted(xp) if xp.ndim == 1 else self.rmatmat_permuted(xp)
        y = self.unpermute(yp)
        if on_dev:
            return y.to(orig_dtype if orig_dtype.is_floating_point else torch.float64)
        return y.cpu().numpy().astype(self.dtype, copy=False)

    def rmatvec(self, x):
        return self._rmatvec(x)

    def rmatmat(self, X):
        return self._rmatvec(X)

    def __matmul__(self, x):
        if isinstance(x, torch.Tensor):
            return self._matmat(x)
        if isinstance(x, np.ndarray) and x.ndim in (1, 2):
            if x.shape[0] != self.shape[1]:
                raise ValueError("dimension mismatch")
            return self._matmat(x)
        return super().__matmul__(x)

    def matvec(self, x):
        return self._matmat(x)

    def matmat(self, X):
        return self._matmat(X)

    def dot(self, x):
        return self @ x

    # -- reference API: size / structure ---------------------------------
    # The block tree of the reference (compressed_form_factors.py:808-873)
    # is answered from the plan arrays through _HostTree: which blocks the
    # materialised tree holds, their kinds after the reference's
    # post-processing, heights, bytes and depth-first order.
    @property
    def nbytes(self):
        return int(self._host_tree.nbytes[0])

    @property
    def device_nbytes(self):
        """Bytes held on the device by the operator (pool unless offloaded,
        panels, tensor-core operands, tables)."""
        ts = [self._pool, *self._dev.values(), *self._build_dev.values(),
              *self.__dict__.get("_tc", {}).values()]
        for pnl, vp in self._panels.values():
            ts += [pnl, vp]
        return sum(t.numel() * t.element_size() for t in ts
                   if isinstance(t, torch.Tensor) and t.is_cuda)

    @property
    def depth(self):
        return int(self._host_tree.height[0])

    @property
    def _host_tree(self):
        ht = self.__dict__.get("_host_tree_cache")
        if ht is None:
            ht = _HostTree(self)
            self._host_tree_cache = ht
        return ht

    @property
    def _root(self):
        if self._root_cache is None:
            self._root_cache = self._block_view(0)
        return self._root_cache

    def _check_depth(self, depth):
        if depth > self.depth:
            raise Exception('specified depth (%d) exceeds tree depth (%d)' % (depth, self.depth))

    def _check_row(self, row_ind):
        if not (0 <= row_ind < self.num_faces):
            raise Exception('row_ind (== %d) should be in range [0, %d)' % (row_ind, self.num_faces))

    def get_blocks_at_depth(self, depth):
        """The blocks of the tree at `depth`, depth-first (the root alone at
        depth 0 or when it is a leaf)."""
        self._check_depth(depth)
        ht = self._host_tree
        if depth == 0 or ht.kind[0] != NODE:
            yield self._root
            return
        for b in ht.in_order(ht.alive & (self._depth == depth)):
            yield self._block_view(b)

    def get_row_inds_at_depth(self, depth):
        """Row index sets down the diagonal: every diagonal block at `depth`,
        and every diagonal leaf above it, depth-first."""
        self._check_depth(depth)
        if depth == 0:
            yield np.arange(self.num_faces)
            return
        ht = self._host_tree
        d = self._depth
        sel = ht.alive & ht.diagonal & (d >= 1) & ((d == depth) | ((d < depth) & ht.is_leaf))
        for b in ht.in_order(sel):
            yield self._tree.ref_indices(self._rows[b])

    def get_row_blocks(self, row_ind):
        """The leaves of the tree whose rows hold facet `row_ind`, depth-first."""
        self._check_row(row_ind)
        ht = self._host_tree
        if ht.kind[0] != NODE:
            yield self._root
            return
        for b in ht.in_order(ht.alive & ht.is_leaf & ht.holds_row(row_ind)):
            yield self._block_view(b)

    def get_col_inds_for_row(self, row_ind):
        """Column index sets of the leaves get_row_blocks(row_ind) yields."""
        self._check_row(row_ind)
        ht = self._host_tree
        if ht.kind[0] != NODE:
            yield np.arange(self.num_faces)
            return
        for b in ht.in_order(ht.alive & ht.is_leaf & ht.holds_row(row_ind)):
            yield self._tree.ref_indices(self._cols[b])

    def _with_root(self, root):
        return _HostOperator(self, root)

    def get_individual_block(self, i, j):
        """The operator with every top-level block but (i, j) set to zero
        (as the reference's docstring states; a host-side operator)."""
        return self._with_root(self._root.get_individual_block(i, j))

    def get_diag_blocks(self):
        return self._with_root(self._root.get_diag_blocks())

    def get_off_diag_blocks(self):
        return self._with_root(self._root.get_off_diag_blocks())

    def toarray(self):
        n = self.num_faces
        eye = np.eye(n, dtype=self.dtype)
        return np.asarray(self @ eye)

    def tocsr(self):
        return scipy.sparse.csr_matrix(self.toarray())

    # -- persistence -------------------------------------------------------
    def save(self, path):
        with open(path, 'wb') as f:
            pickle.dump(self, f)

    @staticmethod
    def from_file(path):
        with open(path, 'rb') as f:
            return pickle.load(f)

    _DEV_DICTS = ("_dev", "_dev_tc", "_build_dev", "_nf")

    def __getstate__(self):
        st = dict(self.__dict__)
        st["_root_cache"] = None
        st.pop("_host_tree_cache", None)
        st.pop("_transposed", None)
        st["_desc"] = None
        st["_desc_tc"] = None
        st["_desc_tc64"] = None
        st["_desc_tc_items"] = None
        st["_desc128"] = None
        st["_dev128"] = None
        st["_desc256"] = None
        st["_dev256"] = None
        st["_panels"] = {}
        st["_tc"] = {}
        st["_flags_d"] = None
        st.pop("_fgb_adjoint_ops", None)
        for key in ("_pool", "_perm_d", "_iperm_d"):
            st[key] = st[key].cpu()
        for key in self._DEV_DICTS:
            if st.get(key) is not None:
                st[key] = {k: v.cpu() for k, v in st[key].items()}
        tc = st.get("_exact_csr")
        if tc is not None:
            st["_exact_csr"] = {"indptr": tc.indptr.cpu(), "indices": tc.indices.cpu(),
                                "data": tc.data.cpu(), "row_off": tc.row_off,
                                "bits": tc.bits.cpu(), "word_off": tc.word_off}
        return st

    def __setstate__(self, st):
        from .form_factors import TileCSR
        self.__dict__.update(st)
        if "_exact_pos" not in st and "_exact_index" in st:
            self._exact_pos = np.full(len(self._rows), -1, np.int64)
            for b, q in st["_exact_index"].items():
                self._exact_pos[b] = q
        dev = self.shape_model._device
        for key in ("_pool", "_perm_d", "_iperm_d"):
            setattr(self, key, getattr(self, key).to(dev))
        for key in self._DEV_DICTS:
            if getattr(self, key, None) is not None:
                setattr(self, key, {k: v.to(dev) for k, v in getattr(self, key).items()})
        if self._exact_csr is not None:
            dct = self._exact_csr
            self._exact_csr = TileCSR(dct["indptr"].to(dev), dct["indices"].to(dev),
                                      dct["data"].to(dev), dct["row_off"], 0, 0,
                                      dct["bits"].to(dev), dct["word_off"])
        self._desc = self._make_desc(int(self.stats["num_items"]), int(self.stats["num_tiles"]),
                                     int(self.stats["max_group_tiles"]),
                                     int(self._dev["a_woff"][-1].item()))
        self._desc_tc = self._make_desc_tc()
        self._desc_tc64 = self._make_desc_tc(64)
        self._desc_tc_items = self._make_desc_tc_items()

    # -- leaf data for the Python block objects --------------------------
    def _block_view(self, b):
        """The block object of plan block b (its class from the kind the
        materialised tree gives it)."""
        ht = self._host_tree
        tree = self._tree
        shape = (int(tree.size[self._rows[b]]), int(tree.size[self._cols[b]]))
        cls = _LEAF_CLASS.get(int(ht.kind[b]))
        if cls is None:
            if b == 0:
                cls = FormFactorPartitionBlock if self._parts is not None else self._RootBlock
            else:
                cls = FormFactorOctreeBlock if tree.ndim == 3 else FormFactorQuadtreeBlock
        return cls(self, shape, b)

    def _ref_positions(self, b, sub, outer=None):
        """Positions of the rows and columns of block `sub` within those of
        block b, both in the reference's ascending-id order (`outer`: b's
        own index sets, when the caller has them)."""
        t = self._tree
        Ib, Jb = outer if outer is not None else (t.ref_indices(self._rows[b]),
                                                 t.ref_indices(self._cols[b]))
        ri = np.searchsorted(Ib, t.ref_indices(self._rows[sub]))
        ci = np.searchsorted(Jb, t.ref_indices(self._cols[sub]))
        return ri, ci

    def _block_matrix(self, b):
        """Dense array of block b (an exact leaf or a block the tree holds
        as one dense / sparse leaf), rows and columns in ascending-id order:
        the exact leaves under b placed at their positions."""
        ht = self._host_tree
        m, n = (int(self._tree.size[self._rows[b]]), int(self._tree.size[self._cols[b]]))
        mat = np.zeros((m, n), dtype=self.dtype)
        outer = (self._tree.ref_indices(self._rows[b]), self._tree.ref_indices(self._cols[b]))
        for leaf in ht.plan_leaves_under(b):
            if self._exact_pos[leaf] < 0 or self._leaf_nnz[leaf] == 0:
                continue
            ri, ci = self._ref_positions(b, leaf, outer)
            mat[np.ix_(ri, ci)] = self._leaf_dense(leaf)
        return mat

    def _leaf_dense(self, b):
        """Dense (m x n) array of an exact leaf in the shape dtype, rows and
        columns in the reference's ascending-id order."""
        tree = self._tree
        m, n = int(tree.size[self._rows[b]]), int(tree.size[self._cols[b]])
        q = int(self._exact_pos[b])
        mat = np.zeros((m, n), dtype=self.dtype)
        tc = self._exact_csr
        if q < 0 or tc is None:
            return mat
        r0, r1 = int(tc.row_off[q]), int(tc.row_off[q + 1])
        ip = tc.indptr[r0:r1 + 1].cpu().numpy()
        a, bnd = int(ip[0]), int(ip[-1])
        cols = tc.indices[a:bnd].cpu().numpy()
        vals = tc.data[a:bnd].cpu().numpy()
        rows = np.repeat(np.arange(m), np.diff(ip))
        mat[rows, cols] = vals
        ri = np.argsort(tree.indices(self._rows[b]), kind="stable")
        ci = np.argsort(tree.indices(self._cols[b]), kind="stable")
        return mat[ri][:, ci]

    def _leaf_lowrank(self, b):
        tree = self._tree
        m, n = tree.size[self._rows[b]], tree.size[self._cols[b]]
        k = int(self._rank[b])
        q = np.where(self._lr_blocks == b)[0]
        if k == 0 or q.size == 0:
            return np.zeros((m, 0)), np.zeros(0), np.zeros((0, n))
        q = int(q[0])
        woff = int(self._lr_u[q])
        voff = int(self._lr_v[q])
        Ut = self._pool[woff:woff + k * m].cpu().numpy().reshape(k, m).astype(np.float64)
        Vt = self._pool[voff:voff + k * n].cpu().numpy().reshape(k, n).astype(np.float64)
        # orthogonalise to the reference's (u, s, vt) form
        ri = np.argsort(tree.indices(self._rows[b]), kind="stable")
        ci = np.argsort(tree.indices(self._cols[b]), kind="stable")
        Qu, Ru = np.linalg.qr(Ut.T[ri])
        Qv, Rv = np.linalg.qr(Vt.T[ci])
        W, s, Xt = np.linalg.svd(Ru @ Rv.T)
        return Qu @ W, s, Xt @ Qv.T


# ------------------------------------------------ host view of the tree --
class _HostTree:
    """The materialised block tree of an operator, derived from its plan
    arrays level by level (no recursion over block objects).

    The plan's leaves are the device's leaves.  On top of them the tree
    follows the reference's post-processing of make_block
    (compressed_form_factors.py:313-377), bottom-up: a block whose exact
    leaves hold no nonzero is a zero block; a block made only of exact
    leaves is one sparse leaf when its CSR takes no more bytes than its
    children; else all-dense children become one dense leaf and all-sparse
    (or zero) children one sparse leaf.  The root keeps its children.

    Per block: ``kind`` (after that processing), ``alive`` (the block is in
    the tree: every ancestor is an interior block), ``height`` (0 for
    leaves), ``nbytes`` (the reference's byte count), ``pre`` (depth-first
    preorder position) and ``span`` (blocks in its subtree)."""

    def __init__(self, op):
        tree = op._tree
        rows, cols = op._rows, op._cols
        nb = rows.size
        self.op = op
        m = tree.size[rows].astype(np.int64)
        n = tree.size[cols].astype(np.int64)
        isz = np.dtype(op.dtype).itemsize
        kind = op._kind.astype(np.int64).copy()
        rank = op._rank.astype(np.int64)
        kind[(kind == LEAF_LOWRANK) & (rank == 0)] = LEAF_ZERO
        nnz = op._leaf_nnz.astype(np.int64).copy()
        has_lr = kind == LEAF_LOWRANK
        nbytes = np.zeros(nb, np.int64)
        for k_, per in ((LEAF_DENSE, m * n * isz), (LEAF_SPARSE, nnz * isz),
                        (LEAF_LOWRANK, (m + n + 1) * rank * 8)):
            sel = kind == k_
            nbytes[sel] = per[sel]
        self.nkids = np.zeros(nb, np.int64)
        interior = np.flatnonzero(kind == NODE)
        self.nkids[interior] = tree.nch ** 2
        if kind[0] == NODE:
            self.nkids[0] = int(np.prod(op._root_bshape))
        height = np.zeros(nb, np.int64)
        depth = op._depth
        for d in np.unique(depth[interior])[::-1]:
            at_d = interior[depth[interior] == d]
            for k_ in np.unique(self.nkids[at_d]):
                g = at_d[self.nkids[at_d] == k_]
                kids = op._child0[g][:, None] + np.arange(k_)
                kk = kind[kids]
                any_lr = has_lr[kids].any(1)
                tot = nnz[kids].sum(1)
                child_bytes = nbytes[kids].sum(1) + 8 * (m[g] + n[g])
                csr_bytes = tot * (isz + 4) + (m[g] + 1) * 4
                may = (g != 0) & ~any_lr
                zero = may & (tot == 0)
                csr = may & ~zero & (csr_bytes <= child_bytes)
                rest = (g != 0) & ~zero & ~csr
                dense = rest & (kk == LEAF_DENSE).all(1)
                sparse = rest & ~dense & np.isin(kk, (LEAF_SPARSE, LEAF_ZERO)).all(1)
                new = np.full(g.size, NODE, np.int64)
                new[zero] = LEAF_ZERO
                new[csr | sparse] = LEAF_SPARSE
                new[dense] = LEAF_DENSE
                kind[g] = new
                nnz[g] = tot
                has_lr[g] = any_lr
                nbytes[g] = np.select([new == NODE, new == LEAF_DENSE, new == LEAF_SPARSE],
                                      [child_bytes, m[g] * n[g] * isz, tot * isz], 0)
                height[g] = np.where(new == NODE, 1 + height[kids].max(1), 0)
        self.kind, self.nbytes, self.height = kind, nbytes, height
        self.is_leaf = kind != NODE
        self.diagonal = rows == cols
        # blocks in the tree, subtree sizes and preorder positions
        parent = op._parent
        alive = np.zeros(nb, bool)
        alive[0] = True
        levels = [np.flatnonzero(depth == d) for d in range(int(depth.max()) + 1)]
        for ids in levels[1:]:
            p = parent[ids]
            alive[ids] = alive[p] & (kind[p] == NODE)
        self.alive = alive
        span = np.where(alive, 1, 0).astype(np.int64)
        for ids in levels[:0:-1]:
            ids = ids[alive[ids]]
            np.add.at(span, parent[ids], span[ids])
        pre = np.full(nb, -1, np.int64)
        pre[0] = 0
        for ids in levels[:-1]:
            ids = ids[alive[ids] & (kind[ids] == NODE)]
            for k_ in np.unique(self.nkids[ids]):
                g = ids[self.nkids[ids] == k_]
                kids = op._child0[g][:, None] + np.arange(k_)
                before = np.cumsum(span[kids], 1) - span[kids]
                pre[kids] = pre[g][:, None] + 1 + before
        self.span, self.pre = span, pre

    def in_order(self, mask):
        """Block ids selected by `mask`, in depth-first order."""
        ids = np.flatnonzero(mask)
        return ids[np.argsort(self.pre[ids], kind="stable")]

    def holds_row(self, row_ind):
        """Blocks whose row cluster holds facet `row_ind`."""
        tree = self.op._tree
        if getattr(self, "_iperm", None) is None:
            self._iperm = np.empty_like(tree.perm)
            self._iperm[tree.perm] = np.arange(tree.perm.size)
        p = int(self._iperm[row_ind])
        r = self.op._rows
        return (tree.start[r] <= p) & (p < tree.start[r] + tree.size[r])

    def subtree(self, b):
        """Blocks of the materialised tree under b (b first), depth-first."""
        lo, hi = self.pre[b], self.pre[b] + self.span[b]
        return self.in_order(self.alive & (self.pre >= lo) & (self.pre < hi))

    def plan_leaves_under(self, b):
        """The plan's own leaves under block b (whatever the tree made of
        them): walk the plan's child ranges down from b."""
        op = self.op
        out, front = [], np.array([b], np.int64)
        while front.size:
            node = op._kind[front] == NODE
            out.append(front[~node])
            inner = front[node]
            if not inner.size:
                break
            nk = np.where(inner == 0, int(np.prod(op._root_bshape)), op._tree.nch ** 2)
            front = np.concatenate([op._child0[i] + np.arange(k) for i, k in zip(inner, nk)])
        return np.concatenate(out) if out else np.zeros(0, np.int64)


class _HostOperator(scipy.sparse.linalg.LinearOperator):
    """A CompressedFormFactorMatrix with its top-level blocks replaced
    (get_diag_blocks and friends): products on the host, through the
    given root block."""

    def __init__(self, op, root):
        self._op = op
        self._root = root
        self.shape_model = op.shape_model

    @property
    def shape(self):
        return self._op.shape

    @property
    def dtype(self):
        return self._op.dtype

    @property
    def ndim(self):
        return 2

    def _matmat(self, x):
        return self._root @ x

    def _matvec(self, x):
        return self._root @ x

    def __matmul__(self, x):
        return self._root @ x


# ------------------------------------------------------- block classes --
class CompressedFormFactorBlock:
    """A block of a CompressedFormFactorMatrix (compressed_form_factors.py:35):
    a view of block b of the operator's plan, or (b < 0) a block made on
    the host (the zero blocks of get_diag_blocks and friends)."""

    def __init__(self, root, shape, b=-1):
        self._root = root
        self.shape = (int(shape[0]), int(shape[1]))
        self._b = b

    @property
    def dtype(self):
        return self._root.dtype

    @property
    def size(self):
        return self.shape[0] * self.shape[1]

    @property
    def root(self):
        return self._root

    @property
    def nbytes(self):
        return int(self._root._host_tree.nbytes[self._b]) if self._b >= 0 else 0

    @property
    def depth(self):
        return int(self._root._host_tree.height[self._b]) if self._b >= 0 else 0

    def __matmul__(self, x):
        return self._matmat(np.asarray(x))


class FormFactorLeafBlock(CompressedFormFactorBlock):
    is_leaf = True
    is_empty_leaf = False

    def get_blocks_at_depth(self, depth):
        if depth == 0:
            yield self

    _get_blocks_at_depth = get_blocks_at_depth

    def _matmat(self, x):
        return self._mat @ x


class FormFactorNullBlock(FormFactorLeafBlock):
    """A block with no rows or no columns (the plan gives such blocks to
    FormFactorZeroBlock; kept for the reference's API)."""
    is_empty_leaf = True

    def __init__(self, root, shape, b=-1):
        if shape[0] != 0 and shape[1] != 0:
            raise RuntimeError('a null block must have a degenerate shape')
        super().__init__(root, shape, b)

    def _matmat(self, x):
        if self.shape[1] != x.shape[0]:
            raise ValueError('multiplying null block with matrix with wrong shape')
        return np.empty((self.shape[0],) + x.shape[1:], dtype=self.dtype)

    def is_dense(self):
        return True

    def is_sparse(self):
        return True

    @property
    def _mat(self):
        return np.empty(self.shape, dtype=self.dtype)


class FormFactorZeroBlock(FormFactorLeafBlock):
    is_empty_leaf = True

    def _matmat(self, x):
        return np.zeros((self.shape[0],) + x.shape[1:], dtype=self.dtype)

    def is_dense(self):
        return False

    def is_sparse(self):
        return True

    @property
    def _mat(self):
        return np.zeros(self.shape, self.dtype)

    def tocsr(self):
        return scipy.sparse.csr_matrix(self.shape, dtype=self.dtype)


class FormFactorDenseBlock(FormFactorLeafBlock):
    @property
    def _mat(self):
        got = self.__dict__.get("_dense")
        if got is None:
            got = self._dense = self._root._block_matrix(self._b)
        return got

    def toarray(self):
        return self._mat

    def is_dense(self):
        return True

    def is_sparse(self):
        return False


class FormFactorSparseBlock(FormFactorLeafBlock):
    def is_dense(self):
        return False

    def is_sparse(self):
        return True

    def _matmat(self, x):
        return np.asarray(self._spmat @ x)


class FormFactorCsrBlock(FormFactorSparseBlock):
    @property
    def _spmat(self):
        got = self.__dict__.get("_csr")
        if got is None:
            got = self._csr = scipy.sparse.csr_matrix(self._root._block_matrix(self._b))
        return got

    def tocsr(self):
        return self._spmat

    @property
    def _mat(self):
        return self._spmat.toarray()


class FormFactorSvdBlock(FormFactorLeafBlock):
    """Low-rank leaf in the reference's (u, s, vt) form, orthogonalised
    from the stored factors on first use."""

    def _factors(self):
        got = self.__dict__.get("_usv")
        if got is None:
            got = self._usv = self._root._leaf_lowrank(self._b)
        return got

    @property
    def _u(self):
        return self._factors()[0]

    @property
    def _s(self):
        return self._factors()[1]

    @property
    def _vt(self):
        return self._factors()[2]

    @property
    def _k(self):
        return self._s.size

    def _matmat(self, x):
        u, s, vt = self._factors()
        t = vt @ x
        return u @ (s.reshape((-1,) + (1,) * (t.ndim - 1)) * t)

    def is_dense(self):
        return False

    def is_sparse(self):
        return False

    @property
    def _mat(self):
        u, s, vt = self._factors()
        return (u * s) @ vt


_LEAF_CLASS = {LEAF_ZERO: FormFactorZeroBlock, LEAF_DENSE: FormFactorDenseBlock,
               LEAF_SPARSE: FormFactorCsrBlock, LEAF_LOWRANK: FormFactorSvdBlock}


class FormFactorBlockMatrix(CompressedFormFactorBlock):
    """Interior block (compressed_form_factors.py:279-510): its children
    are the plan's child blocks, row-major over (row cluster, column
    cluster); ``_zeroed`` lists children replaced by zero blocks."""
    is_leaf = False
    is_empty_leaf = False
    _zeroed = frozenset()

    def _child_ids(self):
        op = self._root
        return op._child0[self._b] + np.arange(int(op._host_tree.nkids[self._b]))

    @property
    def bshape(self):
        op = self._root
        if self._b == 0:
            return tuple(op._root_bshape)
        return (op._tree.nch, op._tree.nch)

    def _index_sets(self, axis):
        op = self._root
        ids = self._child_ids()
        nr, nc = self.bshape
        first = ids[::nc] if axis == 0 else ids[:nc]
        return [op._ref_positions(self._b, c)[axis] for c in first]

    @property
    def _row_block_inds(self):
        got = self.__dict__.get("_rinds")
        if got is None:
            got = self._rinds = self._index_sets(0)
        return got

    @property
    def _col_block_inds(self):
        got = self.__dict__.get("_cinds")
        if got is None:
            got = self._cinds = self._index_sets(1)
        return got

    @property
    def _blocks(self):
        got = self.__dict__.get("_kids")
        if got is None:
            op = self._root
            nr, nc = self.bshape
            got = np.empty((nr, nc), dtype=object)
            for q, c in enumerate(self._child_ids()):
                i, j = divmod(q, nc)
                got[i, j] = (FormFactorZeroBlock(op, got_shape(op, c)) if (i, j) in self._zeroed
                             else op._block_view(c))
            self._kids = got
        return got

    @property
    def nbytes(self):
        if not self._zeroed:
            return super().nbytes
        # the index arrays and the blocks left in place
        return 8 * (self.shape[0] + self.shape[1]) + sum(
            b.nbytes for b in self._blocks.ravel())

    @property
    def depth(self):
        if not self._zeroed:
            return super().depth
        return 1 + max(b.depth for b in self._blocks.ravel())

    def is_dense(self):
        return all(isinstance(b, FormFactorDenseBlock) for b in self._blocks.ravel())

    def is_sparse(self):
        return all(isinstance(b, (FormFactorSparseBlock, FormFactorZeroBlock))
                   for b in self._blocks.ravel())

    def _get_blocks_at_depth(self, depth):
        """Blocks `depth` levels below this one, depth-first."""
        if depth == 0:
            yield self
            return
        if depth == 1:
            yield from self._blocks.ravel()
            return
        op = self._root
        ht = op._host_tree
        d0 = op._depth[self._b]
        for c in ht.subtree(self._b):
            if op._depth[c] - d0 == depth and not self._under_zeroed(c):
                yield op._block_view(c)

    def _under_zeroed(self, c):
        if not self._zeroed or c == self._b:
            return False
        ht = self._root._host_tree
        nc = self.bshape[1]
        for (i, j) in self._zeroed:
            z = self._root._child0[self._b] + i * nc + j
            if ht.pre[z] <= ht.pre[c] < ht.pre[z] + ht.span[z]:
                return True
        return False

    def _matmat(self, x):
        """y = block @ x: every leaf of the subtree applied once at its rows
        and columns (leaves of zeroed children skipped)."""
        op = self._root
        ht = op._host_tree
        y = np.zeros((self.shape[0],) + x.shape[1:], dtype=np.result_type(self.dtype, x.dtype))
        outer = (op._tree.ref_indices(op._rows[self._b]), op._tree.ref_indices(op._cols[self._b]))
        for c in ht.subtree(self._b):
            if not ht.is_leaf[c] or ht.kind[c] == LEAF_ZERO or self._under_zeroed(c):
                continue
            ri, ci = op._ref_positions(self._b, c, outer)
            y[ri] += op._block_view(c)._matmat(x[ci])
        return y

    def _masked(self, zeroed):
        out = type(self)(self._root, self.shape, self._b)
        out._zeroed = frozenset(zeroed)
        return out

    def get_individual_block(self, i, j):
        """A copy in which every child but (i, j) is a zero block."""
        nr, nc = self.bshape
        return self._masked((a, b) for a in range(nr) for b in range(nc) if (a, b) != (i, j))

    def get_diag_blocks(self):
        nr, nc = self.bshape
        return self._masked((a, b) for a in range(nr) for b in range(nc) if a != b)

    def get_off_diag_blocks(self):
        nr, nc = self.bshape
        return self._masked((a, a) for a in range(min(nr, nc)))


def got_shape(op, b):
    return (int(op._tree.size[op._rows[b]]), int(op._tree.size[op._cols[b]]))


class FormFactor2dTreeBlock(FormFactorBlockMatrix):
    pass


class FormFactorQuadtreeBlock(FormFactor2dTreeBlock):
    """Quadtree interior block (compressed_form_factors.py:622-641)."""


class FormFactorOctreeBlock(FormFactor2dTreeBlock):
    """Octree interior block (compressed_form_factors.py:643-658)."""


class FormFactorPartitionBlock(FormFactorBlockMatrix):
    """Root block split into user-given parts of the facets
    (compressed_form_factors.py:660-698).  Build it with
    ``CompressedFormFactorMatrix(shape_model, RootBlock=FormFactorPartitionBlock,
    parts=[I_0, I_1, ...], ChildBlock=FormFactorQuadtreeBlock)``: the parts
    must be disjoint (the reference's check and message) and, here, cover
    every facet; each part is used in ascending index order.  Like the
    reference's, it reports itself as an empty leaf."""
    is_empty_leaf = True


class CompressedKernelMatrix(scipy.sparse.linalg.LinearOperator):
    """(I - rho F) and its transpose product (compressed_form_factors.py:875-913)."""

    def __init__(self, form_factor_matrix, rho, albedo_placement='right'):
        self.form_factor_matrix = form_factor_matrix
        if not (0 < rho <= 1):
            raise ValueError('need 0 < rho <= 1')
        self.rho = rho
        if albedo_placement not in {'left', 'right'}:
            raise ValueError('albedo_placement must be "left" or "right"')
        self.albedo_placement = albedo_placement

    @property
    def shape(self):
        return self.form_factor_matrix.shape

    @property
    def dtype(self):
        return self.form_factor_matrix.dtype

    @property
    def ndim(self):
        return 2

    def _matvec(self, x):
        y = x.copy() if not isinstance(x, torch.Tensor) else x.clone()
        if self.albedo_placement == 'left':
            y -= self.rho * (self.form_factor_matrix @ x)
        elif self.albedo_placement == 'right':
            y -= self.form_factor_matrix @ (self.rho * x)
        else:
            raise RuntimeError('albedo_placement must be "left" or "right"')
        return y

    def _matmat(self, X):
        return self._matvec(X)

    def __matmul__(self, x):
        return self._matvec(x)

    # direct methods: scipy's LinearOperator dispatch needs state that this
    # class (like the reference's, which never calls LinearOperator.__init__)
    # does not set up
    def matvec(self, x):
        return self._matvec(x)

    def rmatvec(self, x):
        return self._rmatvec(x)

    def _rmatvec(self, x):
        y = x.copy() if not isinstance(x, torch.Tensor) else x.clone()
        FT = _transpose_product(self.form_factor_matrix)
        if self.albedo_placement == 'left':
            y -= FT(self.rho * x)
        elif self.albedo_placement == 'right':
            y -= self.rho * FT(x)
        else:
            raise RuntimeError('albedo_placement must be "left" or "right"')
        return y


def _transpose_product(F):
    """x -> x @ F (i.e. F^T x) for scipy matrices, dense arrays and the
    compressed operator (its transposed panel product on the device)."""
    def apply(x):
        if isinstance(F, CompressedFormFactorMatrix):
            return F._rmatvec(x)
        return np.asarray(x @ F).ravel() if np.ndim(x) == 1 else np.asarray(x @ F)
    return apply
