"""GPU: the block-tree introspection of the compressed operator
(CompressedFormFactorMatrix.get_blocks_at_depth, get_row_inds_at_depth,
get_row_blocks, get_col_inds_for_row, depth, nbytes, _root._blocks) against
the reference's own answers on the same matrices (tests/golden/tree.npz,
made by tests/golden/make_golden.py from src/flux/compressed_form_factors.py:
808-847), and save / from_file round trips of the operator."""
import numpy as np
import pytest
import torch

from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                  FormFactorOctreeBlock, FormFactorQuadtreeBlock)
from fluxpy_gb300.form_factors import get_form_factor_matrix

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["octsphere", "crater_quad1", "crater_quad2", "crater_quad3"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN / "tree.npz")


@pytest.fixture(scope="module")
def ffref():
    return np.load(GOLDEN / "ffref.npz")


_ops = {}


def _operator(case, ffref):
    if case not in _ops:
        if case == "octsphere":
            sm = gshape.EmbreeTrimeshShapeModel(ffref["octsphere_V"], ffref["octsphere_F"],
                                                N=ffref["octsphere_N"].copy())
            _ops[case] = CompressedFormFactorMatrix(sm, tol=0, max_depth=1, force_max_depth=True,
                                                    RootBlock=FormFactorOctreeBlock)
        else:
            depth = int(case[-1])
            V, F = terrain.spherical_crater()
            sm = gshape.EmbreeTrimeshShapeModel(V, F)
            _ops[case] = CompressedFormFactorMatrix(sm, tol=0, max_depth=depth,
                                                    RootBlock=FormFactorQuadtreeBlock,
                                                    min_size=4096)
    return _ops[case]


def _walk(block, depth):
    """Blocks `depth` levels below `block` through the materialised
    _blocks arrays (an independent path through the same tree)."""
    if depth == 0:
        return [block]
    if block.is_leaf:
        return []
    out = []
    for b in block._blocks.ravel():
        out += _walk(b, depth - 1)
    return out


@pytest.mark.parametrize("case", CASES)
def test_tree_introspection_matches_reference(case, golden, ffref):
    FF = _operator(case, ffref)
    g = {k[len(case) + 1:]: golden[k] for k in golden.files if k.startswith(case + "_")}
    assert FF.depth == int(g["depth"])
    assert FF.nbytes == int(g["nbytes"])
    kids = FF._root._blocks.ravel()
    assert [type(b).__name__ for b in kids] == list(g["root_types"])
    assert [b.nbytes for b in kids] == list(g["root_nbytes"])
    for d in range(FF.depth + 1):
        blocks = list(FF.get_blocks_at_depth(d))
        if f"bad{d}_types" in g:
            assert [type(b).__name__ for b in blocks] == list(g[f"bad{d}_types"])
            assert [b.shape for b in blocks] == [tuple(s) for s in g[f"bad{d}_shapes"]]
            assert [b.nbytes for b in blocks] == list(g[f"bad{d}_nbytes"])
        else:
            # the reference raises AttributeError here (its leaves lack
            # _get_blocks_at_depth); the answer must be the tree's blocks at
            # that depth, depth-first
            assert str(g[f"bad{d}_error"]) == "AttributeError"
            want = _walk(FF._root, d)
            assert [(type(b).__name__, b.shape) for b in blocks] == \
                [(type(b).__name__, b.shape) for b in want]
        sets = list(FF.get_row_inds_at_depth(d))
        assert [len(x) for x in sets] == list(g[f"rid{d}_len"])
        assert np.array_equal(np.concatenate(sets), g[f"rid{d}"])
    with pytest.raises(Exception, match="exceeds tree depth"):
        list(FF.get_blocks_at_depth(FF.depth + 1))
    for i, r in enumerate(g["rows"]):
        blocks = list(FF.get_row_blocks(int(r)))
        assert [type(b).__name__ for b in blocks] == list(g[f"rb{i}_types"])
        assert [b.shape for b in blocks] == [tuple(s) for s in g[f"rb{i}_shapes"]]
        sets = list(FF.get_col_inds_for_row(int(r)))
        assert [len(x) for x in sets] == list(g[f"ci{i}_len"])
        assert np.array_equal(np.concatenate(sets), g[f"ci{i}"])
    with pytest.raises(Exception, match="should be in range"):
        list(FF.get_row_blocks(FF.num_faces))


@pytest.mark.parametrize("case", ["crater_quad3"])
def test_materialised_tree_products(case, ffref):
    FF = _operator(case, ffref)
    Fx = get_form_factor_matrix(FF.shape_model)
    x = np.random.default_rng(0).uniform(0, 1, FF.num_faces)
    y = Fx @ x
    assert np.abs(FF._root @ x - y).max() <= 1e-12 * np.abs(y).max()
    # diagonal + off-diagonal parts add up to the whole
    yd = FF.get_diag_blocks() @ x
    yo = FF.get_off_diag_blocks() @ x
    assert np.abs(yd + yo - y).max() <= 1e-12 * np.abs(y).max()
    # one top-level block (i, j): its rows and columns only
    i, j = 1, 2
    yi = FF.get_individual_block(i, j) @ x
    I = FF._root._row_block_inds[i]
    J = FF._root._col_block_inds[j]
    want = np.zeros_like(y)
    want[I] = Fx[I][:, J] @ x[J]
    assert np.abs(yi - want).max() <= 1e-12 * np.abs(y).max()


def test_save_from_file_round_trip(tmp_path):
    """pickle save / from_file (compressed_form_factors.py:748-751,
    801-803): the reloaded operator multiplies like the original in every
    precision, including rebuilt tensor-core operands, and keeps its tree."""
    V, F = terrain.fbm_terrain(n=40, seed=6, n_craters=3)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, RootBlock=FormFactorOctreeBlock,
                                    dtype=np.float32)
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, sm.num_faces)
    X = torch.as_tensor(rng.uniform(0, 1, (sm.num_faces, 16)), dtype=torch.float32,
                        device="cuda")
    y0 = FF @ x
    Xp = FF.permute(X).contiguous()
    Y0 = FF.matmat_permuted(Xp, "bf16").clone()
    path = tmp_path / "FF.bin"
    FF.save(path)
    G = CompressedFormFactorMatrix.from_file(path)
    assert np.array_equal(G @ x, y0)
    assert torch.equal(G.matmat_permuted(Xp, "bf16"), Y0)
    assert G.depth == FF.depth and G.nbytes == FF.nbytes
    assert [type(b).__name__ for b in G._root._blocks.ravel()] == \
        [type(b).__name__ for b in FF._root._blocks.ravel()]
