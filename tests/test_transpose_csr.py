"""CPU: the transposition of the exact leaves' tile CSR (rows and columns
local to each leaf, visible-pair bitmask) used to build the transposed
operator, against scipy's transposes leaf by leaf, in one chunk and in
several."""
import numpy as np
import pytest
import scipy.sparse
import torch

from fluxpy_gb300.compressed_form_factors import _transpose_exact_csr
from fluxpy_gb300.form_factors import TileCSR


def _leaves(seed):
    rng = np.random.default_rng(seed)
    ms = rng.integers(1, 90, 25)
    ns = rng.integers(1, 90, 25)
    mats = [scipy.sparse.random(m, n, density=rng.uniform(0, 0.4), random_state=rng,
                                format="csr") for m, n in zip(ms, ns)]
    indptr, indices, data, row_off, bits, word_off = [0], [], [], [0], [], [0]
    for A in mats:
        base = indptr[-1]
        indptr += list(base + A.indptr[1:])
        indices += list(A.indices)
        data += list(A.data)
        row_off.append(row_off[-1] + A.shape[0])
        wpr = (A.shape[1] + 31) // 32
        w = np.zeros(A.shape[0] * wpr, np.int64)
        for r in range(A.shape[0]):
            for c in A.indices[A.indptr[r]:A.indptr[r + 1]]:
                w[r * wpr + int(c) // 32] |= 1 << (int(c) % 32)
        bits += list(w)
        word_off.append(word_off[-1] + w.size)
    bits = np.array(bits, np.int64)
    bits = np.where(bits >= 2**31, bits - 2**32, bits).astype(np.int32)
    t = TileCSR(torch.tensor(indptr, dtype=torch.int64), torch.tensor(indices, dtype=torch.int32),
                torch.tensor(data, dtype=torch.float64), np.array(row_off), 0, 0,
                torch.tensor(bits), np.array(word_off))
    return mats, ms, ns, t


@pytest.mark.parametrize("chunk", [10**9, 37])
def test_transpose_tile_csr(chunk):
    mats, ms, ns, t = _leaves(3)
    tt = _transpose_exact_csr(t, ms, ns, chunk_nnz=chunk)
    assert np.array_equal(tt.row_off, np.concatenate([[0], np.cumsum(ns)]))
    bits = tt.bits.numpy().astype(np.int64) & 0xffffffff
    for q, A in enumerate(mats):
        At = A.T.tocsr()
        At.sort_indices()
        r0, r1 = tt.row_off[q], tt.row_off[q + 1]
        ip = tt.indptr[r0:r1 + 1].numpy()
        assert np.array_equal(ip - ip[0], At.indptr)
        assert np.array_equal(tt.indices[ip[0]:ip[-1]].numpy(), At.indices)
        assert np.array_equal(tt.data[ip[0]:ip[-1]].numpy(), At.data)
        wpr = (A.shape[0] + 31) // 32
        w = bits[tt.word_off[q]:tt.word_off[q + 1]].reshape(A.shape[1], wpr)
        for r in range(At.shape[0]):
            cols = At.indices[At.indptr[r]:At.indptr[r + 1]]
            want = np.zeros(wpr, np.int64)
            for c in cols:
                want[int(c) // 32] |= 1 << (int(c) % 32)
            assert np.array_equal(w[r], want), (q, r)
