"""CPU: the vectorised block planner (_plan_blocks in
compressed_form_factors.py) builds exactly the block tree of the per-block
loop it replaced (restated below: the decisions of make_block,
src/flux/compressed_form_factors.py:285-386, with ACA for admissible
blocks), with the same block ids, for trees with and without a partition
root, with and without compression, depth limits and forced depth.  ACA is
replaced by a deterministic stand-in that accepts or rejects blocks."""
import numpy as np
import pytest
import torch

from fluxpy_gb300 import terrain
from fluxpy_gb300.compressed_form_factors import (LEAF_LOWRANK, LEAF_ZERO, NODE, ClusterTree,
                                                  _admissible_blocks, _bbox3, _plan_blocks)


def fake_aca(r, c, base):
    """Rank from the cluster ids; -1 / -2 = not compressible (split), -3 =
    store exactly (an exact leaf, never split)."""
    r, c = np.asarray(r), np.asarray(c)
    ranks = ((r * 31 + c * 17) % 8) - 3
    sz = np.where(ranks > 0, ranks * 3, 0)
    offs = base + np.cumsum(sz) - sz
    offs = np.where(ranks >= 0, offs, -1)
    n = int(sz.sum())
    return ranks, offs, (torch.zeros(n) if n else None)


def loop_plan(tree, lo3, hi3, tol, min_size, maxd, force, eta):
    """The per-block breadth-first loop (one block at a time)."""
    rows, cols, parent, kind, child0, depth, rank, pool_off = ([] for _ in range(8))

    def add(r, c, p, d):
        rows.append(r); cols.append(c); parent.append(p); kind.append(-1)
        child0.append(-1); depth.append(d); rank.append(0); pool_off.append(-1)
        return len(rows) - 1

    def split(b, nxt):
        r, c, d = rows[b], cols[b], depth[b]
        kind[b] = NODE
        first = None
        for rc in tree.children[r]:
            for cc in tree.children[c]:
                nb = add(rc, cc, b, d + 1)
                if first is None:
                    first = nb
                nxt.append(nb)
        child0[b] = first

    root = add(0, 0, -1, 0)
    kind[root] = NODE
    ch = tree.children[0]
    if ch is None:
        level = [add(0, 0, root, 1)]
    else:
        level = [add(r, c, root, 1) for r in ch for c in ch]
    child0[root] = level[0]
    exact, total = [], 0
    while level:
        cand, nxt = [], []
        for b in level:
            r, c, d = rows[b], cols[b], depth[b]
            m, n = tree.size[r], tree.size[c]
            if m == 0 or n == 0:
                kind[b] = LEAF_ZERO
                continue
            at_max = maxd is not None and d >= maxd
            can = tree.children[r] is not None and tree.children[c] is not None and not at_max
            if force and maxd is not None and not at_max and can:
                split(b, nxt)
                continue
            if m * n < min_size and not force:
                exact.append(b)
                continue
            if tol > 0 and _admissible_blocks(lo3, hi3, np.array([r]), np.array([c]), eta)[0]:
                cand.append(b)
                continue
            if can:
                split(b, nxt)
            else:
                exact.append(b)
        if cand:
            ranks, offs, pool = fake_aca([rows[b] for b in cand], [cols[b] for b in cand], total)
            if pool is not None:
                total += pool.numel()
            for b, k, off in zip(cand, ranks, offs):
                if k >= 0:
                    kind[b], rank[b], pool_off[b] = LEAF_LOWRANK, int(k), int(off)
                elif k == -3:
                    exact.append(b)
                else:
                    r, c, d = rows[b], cols[b], depth[b]
                    at_max = maxd is not None and d >= maxd
                    if tree.children[r] is not None and tree.children[c] is not None and not at_max:
                        split(b, nxt)
                    else:
                        exact.append(b)
        level = nxt
    return dict(rows=rows, cols=cols, parent=parent, kind=kind, child0=child0, depth=depth,
                rank=rank, pool_off=pool_off, exact=exact)


def _trees():
    rng = np.random.default_rng(0)
    P1 = rng.random((3000, 3)) * [1.0, 1.0, 0.3]
    V, F = terrain.fbm_terrain(n=40, seed=1, n_craters=3)
    P2 = V[F].mean(1)
    parts = [np.flatnonzero(P2[:, 0] < P2[:, 0].mean()), np.flatnonzero(P2[:, 0] >= P2[:, 0].mean())]
    return [("random3d", P1, 3, None), ("terrain2d", P2, 2, None), ("terrain3d", P2, 3, None),
            ("partition", P2, 3, parts), ("tiny", P1[:40], 3, None)]


@pytest.mark.parametrize("name,P,ndim,parts", _trees(), ids=[t[0] for t in _trees()])
@pytest.mark.parametrize("tol,min_size,maxd,force", [
    (0.0, 4096, None, False), (1e-5, 4096, None, False), (1e-5, 1024, 3, False),
    (1e-5, 0, None, False), (0.0, 16384, 2, True), (1e-5, 4096, 2, True)])
def test_vectorised_plan_equals_block_loop(name, P, ndim, parts, tol, min_size, maxd, force):
    tree = ClusterTree(P, ndim, leaf_size=64, parts=parts)
    lo3, hi3 = _bbox3(P, tree)
    ref = loop_plan(tree, lo3, hi3, tol, min_size, maxd, force, 1.0)
    got = _plan_blocks(tree, lo3, hi3, tol=tol, min_size=min_size, max_depth=maxd,
                       force_max_depth=force, eta=1.0, run_aca=fake_aca)
    for key in ("rows", "cols", "parent", "kind", "child0", "depth", "rank", "pool_off"):
        assert np.array_equal(got[key], np.asarray(ref[key], np.int64)), key
    assert np.array_equal(np.sort(got["exact"]), np.sort(np.asarray(ref["exact"], np.int64)))
    assert got["exact"].size == len(set(ref["exact"]))


def test_exact_leaf_classification_equals_loop():
    from fluxpy_gb300.compressed_form_factors import (LEAF_DENSE, LEAF_SPARSE,
                                                      _classify_exact, _nbytes_csr)
    rng = np.random.default_rng(3)
    m = rng.integers(1, 200, 5000)
    n = rng.integers(1, 200, 5000)
    nnz = (rng.random(5000) * m * n * rng.random(5000)).astype(np.int64)
    nnz[::7] = 0
    for min_size, isz in ((4096, 8), (16384, 4), (0, 8)):
        got = _classify_exact(nnz, m, n, min_size, isz)
        for q in range(m.size):
            if nnz[q] == 0:
                want = LEAF_ZERO
            elif m[q] * n[q] < min_size and m[q] * n[q] * isz < _nbytes_csr(nnz[q], m[q], isz):
                want = LEAF_DENSE
            else:
                want = LEAF_SPARSE
            assert got[q] == want
