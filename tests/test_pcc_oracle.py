"""CPU: the PCC oracle against the reference's golden files and (when the
reference tree is present) against the reference's own C sources."""
import numpy as np
import pytest

from oracle import pcc as opcc
from tests import pcc_scenario as sc
from tests.conftest import GOLDEN
from fluxpy_gb300.thermal import flux_noatm, setgrid


def test_oracle_reproduces_golden_files():
    golden = np.load(GOLDEN / "pcc_conductionQ.npz")
    z = sc.grid(setgrid)
    w = z.size
    T = np.full((1, w), 210.0)
    ti = np.full(w, 120.0)
    rhoc = np.full(w, 960000.0)
    Qn, q = sc.fluxes(flux_noatm)
    state = {"Qprev": np.array([Qn])}

    def step(i, dt):
        X = q[i:i + 1].copy()
        opcc.step_q(z, dt, state["Qprev"], X, T, ti, rhoc, np.ones(1), np.full(1, 0.2))
        state["Qprev"] = X

    prof, surf = sc.run(step, lambda: T[0].copy(), q)
    sc.check_against_golden(prof, surf, golden)


ZFAC = {40: 1.0817, 60: 1.05, 100: 1.03, 255: 1.01}


def _random_case(rng, n, nz):
    z = np.concatenate([[0.0], setgrid(nz, ZFAC.get(nz, 1.0817), 1.0)])
    w = nz + 1
    ti = np.linspace(55, 400, w)
    rhoc = np.full(w, 1.2e6)
    T = rng.uniform(80, 380, size=(n, w))
    Qprev = rng.uniform(0, 1200, n)
    X = rng.uniform(0, 1200, n)
    X[::7] = 0.0
    emiss = rng.uniform(0.9, 1.0, n)
    Fg = rng.uniform(0, 0.05, n)
    return z, ti, rhoc, T, Qprev, X, emiss, Fg


def test_oracle_matches_reference_c_bitwise():
    if opcc.ref_pcc_lib() is None:
        pytest.skip("reference C sources not available on this machine")
    rng = np.random.default_rng(0)
    z, ti, rhoc, T, Qprev, X, emiss, Fg = _random_case(rng, 300, 40)
    T1 = T.copy()
    T2 = T.copy()
    f1 = opcc.step_q(z, 3600.0, Qprev, X, T1, ti, rhoc, emiss, Fg)
    f2 = opcc.ref_step_q(z, 3600.0, Qprev, X, T2, ti, rhoc, emiss, Fg)
    assert np.array_equal(T1, T2)
    assert np.array_equal(f1, f2)
