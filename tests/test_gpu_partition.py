"""GPU: the partition root block (src/flux/compressed_form_factors.py:660-698):
rows and columns split into user-given parts first, then every (part, part)
block by the child block type; products against the exactly assembled form
factors, and the block structure of the materialised tree."""
import numpy as np
import pytest

from tests.conftest import GOLDEN
from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (
    CompressedFormFactorMatrix, FormFactorOctreeBlock, FormFactorPartitionBlock,
    FormFactorQuadtreeBlock)
from fluxpy_gb300.form_factors import get_form_factor_matrix

pytestmark = pytest.mark.gpu


def _parts(P):
    left = np.flatnonzero(P[:, 0] < 0)
    right = np.flatnonzero(P[:, 0] >= 0)
    return [left, right]


@pytest.mark.parametrize("child", [FormFactorQuadtreeBlock, FormFactorOctreeBlock])
def test_partition_root_exact(child):
    ref = np.load(GOLDEN / "ffref.npz")
    sm = gshape.EmbreeTrimeshShapeModel(ref["crater_V"], ref["crater_F"])
    parts = _parts(sm.P)
    FF = CompressedFormFactorMatrix(sm, tol=0, min_size=1024, RootBlock=FormFactorPartitionBlock,
                                    parts=parts, ChildBlock=child)
    Fx = get_form_factor_matrix(sm)
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, sm.num_faces)
    y = FF @ x
    y_ref = Fx @ x
    assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()
    root = FF._root
    assert isinstance(root, FormFactorPartitionBlock)
    assert root._blocks.shape == (2, 2)
    for got, want in zip(root._row_block_inds, parts):
        assert np.array_equal(got, np.sort(want))
    assert all(not isinstance(b, FormFactorPartitionBlock) for b in root._blocks.flatten())
    # the materialised block tree multiplies like the device operator
    assert np.abs(root @ x - y_ref).max() <= 1e-12 * np.abs(y_ref).max()


def test_partition_root_compressed_and_errors():
    V, F = terrain.fbm_terrain(n=48, seed=5, n_craters=4)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    parts = _parts(sm.P - sm.P.mean(0))
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096,
                                    RootBlock=FormFactorPartitionBlock, parts=parts,
                                    ChildBlock=FormFactorOctreeBlock)
    assert FF.stats["lowrank_blocks"] > 0
    Fx = get_form_factor_matrix(sm)
    x = np.random.default_rng(1).uniform(0, 1, sm.num_faces)
    y_ref = Fx @ x
    assert np.abs(FF @ x - y_ref).max() / np.abs(y_ref).max() < 1e-5
    with pytest.raises(Exception, match="parts must be disjoint"):
        CompressedFormFactorMatrix(sm, RootBlock=FormFactorPartitionBlock,
                                   parts=[parts[0], np.concatenate([parts[1], parts[0][:3]])])
    with pytest.raises(ValueError):
        CompressedFormFactorMatrix(sm, RootBlock=FormFactorPartitionBlock, parts=[parts[0]])
