"""CPU: the host view of the block tree (_HostTree and the introspection
methods of CompressedFormFactorMatrix) against a recursive restatement of
the reference's post-processing and traversals
(src/flux/compressed_form_factors.py:313-377 and 460-510, 808-847) on block
plans made by the planner with a stand-in ACA and stand-in nonzero counts."""
import types

import numpy as np
import pytest

from fluxpy_gb300.compressed_form_factors import (LEAF_DENSE, LEAF_LOWRANK, LEAF_SPARSE,
                                                  LEAF_ZERO, NODE, ClusterTree,
                                                  CompressedFormFactorMatrix,
                                                  FormFactorOctreeBlock, _bbox3, _classify_exact,
                                                  _plan_blocks)
from tests.test_block_plan import _trees, fake_aca


def _fake_operator(P, ndim, parts, tol, min_size, maxd, seed):
    tree = ClusterTree(P, ndim, leaf_size=64, parts=parts)
    lo3, hi3 = _bbox3(P, tree)
    plan = _plan_blocks(tree, lo3, hi3, tol=tol, min_size=min_size, max_depth=maxd,
                        force_max_depth=False, eta=1.0, run_aca=fake_aca)
    op = CompressedFormFactorMatrix.__new__(CompressedFormFactorMatrix)
    op.shape_model = types.SimpleNamespace(dtype=np.float64, num_faces=P.shape[0])
    op._tree = tree
    for key in ("rows", "cols", "parent", "kind", "child0", "depth", "rank"):
        setattr(op, "_" + key, plan[key].copy())
    op._root_bshape = plan["root_bshape"]
    op._parts = parts
    op._RootBlock = FormFactorOctreeBlock
    op._root_cache = None
    rng = np.random.default_rng(seed)
    m = tree.size[op._rows]
    n = tree.size[op._cols]
    nnz = np.zeros(op._rows.size, np.int64)
    ex = plan["exact"]
    # stand-in nonzeros of the exact leaves: zero, sparse or nearly full
    choice = rng.integers(0, 3, ex.size)
    frac = np.where(choice == 0, 0.0, np.where(choice == 1, 0.05, 0.97))
    nnz[ex] = (frac * m[ex] * n[ex]).astype(np.int64)
    op._leaf_nnz = nnz
    op._kind[ex] = _classify_exact(nnz[ex], m[ex], n[ex], min_size, 8)
    return op


def _children(op, b):
    if op._kind[b] != NODE:
        return []
    k = int(np.prod(op._root_bshape)) if b == 0 else op._tree.nch ** 2
    return list(range(op._child0[b], op._child0[b] + k))


def _post(op, b, memo):
    """(kind, nnz, has_lowrank, nbytes, height) of block b after the
    reference's make_block post-processing, recursively."""
    if b in memo:
        return memo[b]
    m, n = int(op._tree.size[op._rows[b]]), int(op._tree.size[op._cols[b]])
    kind = int(op._kind[b])
    if kind != NODE:
        nnz = int(op._leaf_nnz[b])
        if kind == LEAF_LOWRANK and op._rank[b] == 0:
            kind = LEAF_ZERO
        r = int(op._rank[b])
        nbytes = {LEAF_ZERO: 0, LEAF_DENSE: m * n * 8, LEAF_SPARSE: nnz * 8,
                  LEAF_LOWRANK: (m + n + 1) * r * 8}[kind]
        memo[b] = (kind, nnz, kind == LEAF_LOWRANK, nbytes, 0)
        return memo[b]
    kids = [_post(op, c, memo) for c in _children(op, b)]
    nnz = sum(k[1] for k in kids)
    has_lr = any(k[2] for k in kids)
    child_bytes = sum(k[3] for k in kids) + 8 * (m + n)
    height = 1 + max(k[4] for k in kids)
    kind = NODE
    if b != 0:
        if not has_lr and nnz == 0:
            kind = LEAF_ZERO
        elif not has_lr and nnz * 12 + (m + 1) * 4 <= child_bytes:
            kind = LEAF_SPARSE
        elif all(k[0] == LEAF_DENSE for k in kids):
            kind = LEAF_DENSE
        elif all(k[0] in (LEAF_SPARSE, LEAF_ZERO) for k in kids):
            kind = LEAF_SPARSE
    if kind == NODE:
        memo[b] = (NODE, nnz, has_lr, child_bytes, height)
    else:
        nb = {LEAF_ZERO: 0, LEAF_DENSE: m * n * 8, LEAF_SPARSE: nnz * 8}[kind]
        memo[b] = (kind, nnz, has_lr, nb, 0)
    return memo[b]


def _preorder(op, memo):
    """Blocks of the materialised tree, depth-first (recursive)."""
    out = []

    def visit(b):
        out.append(b)
        if memo[b][0] == NODE:
            for c in _children(op, b):
                visit(c)
    visit(0)
    return out


@pytest.mark.parametrize("name,P,ndim,parts", _trees(), ids=[t[0] for t in _trees()])
@pytest.mark.parametrize("tol,min_size,maxd", [(0.0, 4096, None), (1e-5, 4096, None),
                                               (0.0, 1024, 3), (1e-5, 1024, 2)])
def test_host_tree_equals_recursive_restatement(name, P, ndim, parts, tol, min_size, maxd):
    op = _fake_operator(P, ndim, parts, tol, min_size, maxd, seed=len(name))
    ht = op._host_tree
    memo = {}
    _post(op, 0, memo)
    order = _preorder(op, memo)
    alive = np.zeros(op._rows.size, bool)
    alive[order] = True
    assert np.array_equal(ht.alive, alive)
    for b in order:
        kind, _, _, nbytes, height = memo[b]
        assert ht.kind[b] == kind, b
        assert ht.nbytes[b] == nbytes, b
        assert ht.height[b] == height, b
    assert list(ht.in_order(ht.alive)) == order
    assert op.depth == memo[0][4] and op.nbytes == memo[0][3]
    # get_blocks_at_depth: the tree's blocks at that depth, depth-first
    for d in range(op.depth + 1):
        got = [blk._b for blk in op.get_blocks_at_depth(d)]
        want = [b for b in order if op._depth[b] == d] if d else [0]
        assert got == want, d
    # get_row_inds_at_depth: down the diagonal (the reference's recursion)
    tree = op._tree

    def rows_at(b, depth):
        kids = _children(op, b)
        nr = int(round(len(kids) ** 0.5))
        diag = [kids[i * nr + i] for i in range(nr)]
        for c in diag:
            if depth == 1 or memo[c][0] != NODE:
                yield tree.ref_indices(op._rows[c])
            else:
                yield from rows_at(c, depth - 1)
    for d in range(1, op.depth + 1):
        got = list(op.get_row_inds_at_depth(d))
        want = list(rows_at(0, d))
        assert len(got) == len(want)
        assert all(np.array_equal(a, b) for a, b in zip(got, want))
    # get_row_blocks / get_col_inds_for_row for a few facets
    rng = np.random.default_rng(1)
    for f in rng.choice(P.shape[0], 5, replace=False):
        p = int(np.flatnonzero(tree.perm == f)[0])
        want = [b for b in order if memo[b][0] != NODE and b != 0 and
                tree.start[op._rows[b]] <= p < tree.start[op._rows[b]] + tree.size[op._rows[b]]]
        got = [blk._b for blk in op.get_row_blocks(int(f))]
        assert got == want
        cols = list(op.get_col_inds_for_row(int(f)))
        assert all(np.array_equal(c, tree.ref_indices(op._cols[b])) for c, b in zip(cols, want))
        assert np.array_equal(np.sort(np.concatenate(cols)), np.arange(P.shape[0]))


def test_hilbert_index_visits_the_grid_along_the_curve():
    """The Hilbert index of the tile order: order-2 curve visits the 4 x 4
    grid cell by cell (each step to an edge neighbour), order-4 curve is a
    bijection onto 0 .. 255 with unit steps."""
    from fluxpy_gb300.compressed_form_factors import _hilbert_index
    x = np.array([0, 1, 1, 0, 0, 0, 1, 1, 2, 2, 3, 3, 3, 2, 2, 3])
    y = np.array([0, 0, 1, 1, 2, 3, 3, 2, 2, 3, 3, 2, 1, 1, 0, 0])
    assert np.array_equal(_hilbert_index(x, y, order=2), np.arange(16))
    gx, gy = np.meshgrid(np.arange(16), np.arange(16), indexing="ij")
    d = _hilbert_index(gx.ravel(), gy.ravel(), order=4)
    assert np.array_equal(np.sort(d), np.arange(256))
    o = np.argsort(d)
    steps = np.abs(np.diff(gx.ravel()[o])) + np.abs(np.diff(gy.ravel()[o]))
    assert np.all(steps == 1)
