"""CPU: the solve oracle reproduces the reference's own solves
(tests/golden/ffref.npz) given the same form factors."""
import numpy as np

from oracle import solve as osolve
from oracle import vis
from tests.conftest import GOLDEN


def test_oracle_solve_matches_reference():
    ref = np.load(GOLDEN / "ffref.npz")
    V, F = ref["crater_V"], ref["crater_F"]
    P, N, A = vis.geometry(V, F)
    FF = vis.Scene(V, F).ff_csr(P, N, A)
    E = ref["crater_E"]
    B, n = osolve.solve_radiosity(FF, E, 0.12)
    assert n == int(ref["crater_niter"])
    assert np.allclose(B, ref["crater_B"], rtol=1e-10, atol=1e-10)
    T = osolve.steady_state_temp(FF, E, 0.12, 0.95)
    assert np.max(np.abs(T - ref["crater_T"])) < 1e-8
    T2 = osolve.steady_state_temp(FF, ref["crater_E2"], 0.12, 0.95)
    assert np.max(np.abs(T2 - ref["crater_T2"])) < 1e-8
