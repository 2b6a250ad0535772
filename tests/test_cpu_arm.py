"""CPU: the CPU baseline's sample (bench.py _cpu_sample: the oracle's form
factors and insolation of a 64 x 64 fBm terrain) and its Jacobi solves
(oracle/solve.py, one direction per solve to an update of 1e-5 max|E|)
against the reference's own code on the same terrain
(tests/golden/cpuarm.npz, made by tests/golden/make_golden.py from
src/flux/form_factors.py:11-72, shape.py:181-244 and solve.py:36-45): the
same sparsity pattern and lit facets, form factors and insolation to
round-off, the same iteration counts and solutions to round-off, so the timed CPU arm does the
reference's work.  (On the machine that made the fixture the reference's
solve and the oracle's took the same time per solve, to 5 %.)"""
import hashlib

import numpy as np

from tests.conftest import GOLDEN

RHO = 0.12


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_cpu_arm_sample_is_the_references():
    import bench
    g = np.load(GOLDEN / "cpuarm.npz")
    FFc, E = bench._cpu_sample()
    assert FFc.shape[0] == int(g["num_faces"]) and FFc.nnz == int(g["nnz"])
    assert _digest(FFc.indptr.astype(np.int64),
                   FFc.indices.astype(np.int64)) == str(g["pattern_digest"])
    # the oracle's entries and the reference's numpy ones differ in the last bits
    assert np.allclose(FFc @ g["x"], g["Ax"], rtol=1e-13, atol=0)
    assert np.allclose(np.asarray(FFc.sum(1)).ravel(), g["rowsum"], rtol=1e-13, atol=0)
    cols = g["cols"]
    Ec = E[:, cols]
    # insolation: the same lit facets (occlusion), values to round-off (a
    # matrix product here, one dot product per direction there)
    assert np.allclose(Ec.sum(0), g["E_sum"], rtol=1e-13, atol=0)
    assert np.allclose(Ec.max(0), g["E_max"], rtol=1e-13, atol=0)
    Ef = E[:, cols[g["full_cols"]]]
    assert np.array_equal(Ef == 0, g["E"] == 0)
    assert np.allclose(Ef, g["E"], rtol=1e-13, atol=0)
    from oracle import solve as osolve
    for k, c in enumerate(cols):
        e = np.ascontiguousarray(E[:, c])
        B, it = osolve.solve_radiosity(FFc, e, RHO, tol=bench.RTOL * float(np.abs(e).max()))
        assert it == int(g["niter"][k])
        hit = np.flatnonzero(g["full_cols"] == k)
        if hit.size:
            Bref = g["B"][:, hit[0]]
            assert np.abs(B - Bref).max() <= 1e-12 * np.abs(Bref).max()
