"""CPU: the cluster tree follows the reference's octree / quadtree split
rule (oracle/tree.py restates src/flux/octree.py:5-18 and quadtree.py:5-18)."""
import numpy as np
import pytest

from oracle.tree import orthant_order
from fluxpy_gb300 import terrain
from fluxpy_gb300.compressed_form_factors import ClusterTree


@pytest.mark.parametrize("ndim", [2, 3])
def test_tree_matches_reference_rule(ndim):
    rng = np.random.default_rng(ndim)
    for P in (rng.random((3000, 3)), terrain.fbm_terrain(n=40, seed=1, n_craters=3)[0]):
        t = ClusterTree(P, ndim, leaf_size=64)
        stack = [0]
        checked = 0
        while stack:
            node = stack.pop()
            ch = t.children[node]
            if ch is None:
                assert t.size[node] <= 64 or np.all(P[t.indices(node), :ndim] ==
                                                     P[t.indices(node)[0], :ndim])
                continue
            I = t.ref_indices(node)
            ref = [I[x] for x in orthant_order(P[I, :ndim])]
            assert len(ch) == 2**ndim
            for c, r in zip(ch, ref):
                assert np.array_equal(t.ref_indices(c), r)
                stack.append(c)
            checked += 1
        assert checked > 1
        # every node is a contiguous range of the cluster order
        assert np.array_equal(np.sort(t.perm), np.arange(P.shape[0]))


@pytest.mark.parametrize("ndim", [2, 3])
def test_partition_root_children_are_the_parts(ndim):
    """FormFactorPartitionBlock roots (compressed_form_factors.py:660-698):
    the root's children are the given parts, each split below by the
    orthant rule."""
    rng = np.random.default_rng(7)
    P = rng.random((2500, 3))
    parts = [np.flatnonzero(P[:, 0] < 0.3), np.flatnonzero((P[:, 0] >= 0.3) & (P[:, 1] < 0.5)),
             np.flatnonzero((P[:, 0] >= 0.3) & (P[:, 1] >= 0.5))]
    t = ClusterTree(P, ndim, leaf_size=64, parts=parts)
    ch = t.children[0]
    assert len(ch) == len(parts)
    for c, I in zip(ch, parts):
        assert np.array_equal(t.ref_indices(c), np.sort(I))
        sub = t.children[c]
        assert sub is not None and len(sub) == 2**ndim
        ref = [I[x] for x in orthant_order(P[I, :ndim])]
        for s, r in zip(sub, ref):
            assert np.array_equal(t.ref_indices(s), np.sort(r))
    assert np.array_equal(np.sort(t.perm), np.arange(P.shape[0]))
