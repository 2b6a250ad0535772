"""GPU: FP64 rank truncation of the low-rank factors (fgb_recompress_f32)
against the oracle's restatement of the reference's truncation rule
(oracle/truncate.py; src/flux/linalg.py:20-51), and the compressed operator
built with it against the un-truncated one and against the exact dense
form factors."""
import ctypes as C

import numpy as np
import pytest
import torch

from fluxpy_gb300 import _lib, shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (LEAF_LOWRANK, CompressedFormFactorMatrix,
                                                  FormFactorOctreeBlock)
from fluxpy_gb300.form_factors import get_form_factor_matrix
from oracle import truncate as otr

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _block(rng, m, n, k, decay):
    """FP32 factors U (m x k), V (n x k) of a block with singular values
    10^(-decay i), mixed by a random k x k matrix (ACA-like, not orthogonal)."""
    if k == 0:
        return np.zeros((m, 0), np.float32), np.zeros((n, 0), np.float32)
    Q1, _ = np.linalg.qr(rng.standard_normal((m, k)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, k)))
    sv = 3e-6 * 10.0 ** (-decay * np.arange(k))
    M = rng.standard_normal((k, k)) + 2 * np.eye(k)
    U = (Q1 * sv) @ M
    V = Q2 @ np.linalg.inv(M).T
    return U.astype(np.float32), V.astype(np.float32)


CASES = [(40, 30, 0, 0.3), (50, 70, 1, 0.3), (64, 64, 2, 2.0), (200, 150, 3, 3.0),
         (300, 500, 17, 0.37), (129, 257, 32, 0.23), (700, 90, 33, 0.37), (512, 640, 47, 0.15),
         (1000, 1500, 64, 0.37), (2000, 64, 64, 0.05), (333, 444, 9, 1.1)]


def _run(blocks, ranks):
    dev = torch.device("cuda")
    parts, offs = [], []
    o = 0
    for U, V in blocks:
        offs.append(o)
        parts += [U.T.ravel(), V.T.ravel()]
        o += U.size + V.size
    pool = torch.as_tensor(np.concatenate(parts) if o else np.zeros(1, np.float32), device=dev)
    t = lambda a, dt: torch.as_tensor(np.asarray(a, dt), device=dev)
    off_in = t(offs, np.int64)
    rank_in = t(ranks, np.int32)
    m = t([U.shape[0] for U, _ in blocks], np.int32)
    n = t([V.shape[0] for _, V in blocks], np.int32)
    out = torch.full((max(o, 1),), float("nan"), device=dev)
    used = torch.zeros(1, dtype=torch.int64, device=dev)
    rank_out = torch.full((len(blocks),), -9, dtype=torch.int32, device=dev)
    off_out = torch.full((len(blocks),), -9, dtype=torch.int64, device=dev)
    queue = torch.zeros(2, dtype=torch.int32, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("fgb_recompress_f32", _lib.ptr(pool), _lib.ptr(off_in), _lib.ptr(rank_in),
              _lib.ptr(m), _lib.ptr(n), len(blocks), TOL, _lib.ptr(out), out.numel(),
              _lib.ptr(used), _lib.ptr(rank_out), _lib.ptr(off_out), _lib.ptr(queue),
              _lib.ptr(flags), _lib.stream_handle())
    torch.cuda.synchronize()
    return (out.cpu().numpy(), rank_out.cpu().numpy(), off_out.cpu().numpy(),
            int(flags.item()), int(used.item()))


def test_truncation_kernel_matches_the_reference_rule():
    rng = np.random.default_rng(0)
    blocks = [_block(rng, *c) for c in CASES]
    ranks = [c[2] for c in CASES]
    out, r_out, o_out, flags, used = _run(blocks, ranks)
    assert flags == 0
    assert used <= sum(U.size + V.size for U, V in blocks)
    for (U, V), k, r, o in zip(blocks, ranks, r_out, o_out):
        m, n = U.shape[0], V.shape[0]
        s, r_ref, Ar = otr.truncate(U, V, TOL)
        assert r == r_ref, (m, n, k)
        if k == 0:
            continue
        Ut = out[o:o + r * m].reshape(r, m).astype(np.float64)
        Vt = out[o + r * m:o + r * (m + n)].reshape(r, n).astype(np.float64)
        if k == 1:
            # rank-1 blocks are copied as they are
            assert np.array_equal(Ut.T.astype(np.float32), U)
            assert np.array_equal(Vt.T.astype(np.float32), V)
            continue
        A = U.astype(np.float64) @ V.astype(np.float64).T
        err = np.linalg.norm(A - Ut.T @ Vt, 2)
        dropped = s[r] if r < s.size else 0.0
        # the truncation error is the first dropped singular value (plus
        # FP32 rounding of the stored factors)
        assert err <= dropped * (1 + 1e-3) + 2e-6 * s[0], (m, n, k, err / s[0], dropped / s[0])
        # V' has orthonormal columns, U' orthogonal columns of norm sigma_i
        assert np.abs(Vt @ Vt.T - np.eye(r)).max() < 1e-4
        nu = np.linalg.norm(Ut, axis=1)
        assert np.allclose(nu, s[:r], rtol=1e-4, atol=1e-6 * s[0])


def test_failure_codes_pass_through():
    rng = np.random.default_rng(1)
    blocks = [_block(rng, 50, 60, 5, 0.5), _block(rng, 10, 10, 0, 0.5)]
    out, r_out, o_out, flags, _ = _run(blocks, [5, -1])
    assert r_out[1] == -1 and o_out[1] == -1


@pytest.fixture(scope="module")
def terrain64():
    V, F = terrain.fbm_terrain(n=64, seed=1, n_craters=4)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    return sm, get_form_factor_matrix(sm)


def test_truncated_operator_against_untruncated_and_dense(terrain64):
    sm, Fx = terrain64
    kw = dict(tol=TOL, min_size=4096, leaf_size=64, RootBlock=FormFactorOctreeBlock,
              aca_tol=TOL / 10)
    FFt = CompressedFormFactorMatrix(sm, recompress=True, **kw)
    FFa = CompressedFormFactorMatrix(sm, recompress=False, **kw)
    # same blocks; truncation only lowers ranks
    assert np.array_equal(FFt._kind, FFa._kind)
    lr = FFt._kind == LEAF_LOWRANK
    assert np.all(FFt._rank[lr] <= FFa._rank[lr])
    assert FFt.stats["truncated_rank_sum"] <= FFt.stats["aca_rank_sum"]
    # block by block: the truncated factors differ from the ACA factors by
    # at most tol times the block's largest singular value
    tree = FFt._tree
    rng = np.random.default_rng(2)
    for b in rng.choice(np.flatnonzero(lr & (FFt._rank > 0)), 40, replace=False):
        ut, st, vt = FFt._leaf_lowrank(b)
        ua, sa, va = FFa._leaf_lowrank(b)
        At, Aa = (ut * st) @ vt, (ua * sa) @ va
        assert np.linalg.norm(At - Aa, 2) <= 1.05 * TOL * sa[0] + 1e-6 * sa[0]
    # FP64 products against the exact dense form factors
    x = np.random.default_rng(3).uniform(0, 1, sm.num_faces)
    y = Fx @ x
    for FF in (FFt, FFa):
        yc = FF.unpermute(FF.matvec_permuted(FF.permute(torch.as_tensor(x, device="cuda")),
                                             "fp32-fp64")).cpu().numpy()
        assert np.abs(yc - y).max() / np.abs(y).max() < TOL
