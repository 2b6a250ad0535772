"""CPU: the oracle's truncation rule (oracle/truncate.py) against the
reference's estimate_rank semantics (src/flux/linalg.py:20-51): the rank is
the index of the first singular value at or below tol times the largest."""
import numpy as np

from oracle import truncate as otr


def test_truncation_rank_rule():
    s = np.array([1.0, 0.5, 1e-5, 1e-6])
    assert otr.truncation_rank(s, 1e-5) == 2          # 1e-5 / 1 <= tol: dropped
    assert otr.truncation_rank(s, 1e-6) == 3
    assert otr.truncation_rank(s, 1e-7) == 4          # none below: keep all
    assert otr.truncation_rank(np.zeros(3), 1e-5) == 0
    assert otr.truncation_rank(np.array([]), 1e-5) == 0


def test_truncate_error_is_the_first_dropped_singular_value():
    rng = np.random.default_rng(0)
    m, n, k = 120, 90, 12
    Q1, _ = np.linalg.qr(rng.standard_normal((m, k)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, k)))
    sv = 10.0 ** (-np.arange(k) / 1.5)
    M = rng.standard_normal((k, k))
    U = (Q1 * sv) @ M
    V = Q2 @ np.linalg.inv(M).T
    s, r, Ar = otr.truncate(U, V, 1e-5)
    assert r == int(np.sum(sv / sv[0] > 1e-5))
    assert np.allclose(s[:k], sv, rtol=1e-9)
    err = np.linalg.norm(U @ V.T - Ar, 2)
    assert abs(err - sv[r]) <= 1e-9 * sv[0]
