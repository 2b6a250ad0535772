"""GPU parity of the batched conduction kernel (fgb_conduction_*) against the
oracle (bit-exact in FP64) and the reference's golden files."""
import numpy as np
import pytest
import torch

from oracle import pcc as opcc
from tests import pcc_scenario as sc
from tests.conftest import GOLDEN
from tests.test_pcc_oracle import _random_case
from fluxpy_gb300.thermal import PccThermalModel1D, flux_noatm, setgrid

pytestmark = pytest.mark.gpu


def _smooth_if_fine(T, z):
    """On the fine 255-layer grid a random profile makes the Crank-Nicolson
    step ring below zero (the oracle too, which the model would raise on):
    there the profiles relax smoothly from the surface value to 250 K."""
    if z.size <= 101:
        return T
    return T[:, :1] + (250.0 - T[:, :1]) * (1.0 - np.exp(-z[None, :] / 0.05))


@pytest.mark.parametrize("nz", [2, 40, 60, 100, 255])
def test_step_q_bitwise_vs_oracle(nz):
    rng = np.random.default_rng(nz)
    n = 1000
    z, ti, rhoc, T, Qprev, X, emiss, Fg = _random_case(rng, n, nz)
    T_host = T.copy()
    model = PccThermalModel1D(z, T_host, ti, rhoc, emiss, Fg, Qprev, T[:, 0].copy())
    Tref = T.copy()
    Qp = Qprev.copy()
    for step in range(4):
        X = rng.uniform(0, 1200, n)
        X[::11] = 0.0
        fs = opcc.step_q(z, 1800.0 * (step + 1), Qp, X, Tref, ti, rhoc, emiss, Fg)
        model.step(1800.0 * (step + 1), X)
        Qp = X
        assert np.array_equal(model.T, Tref), np.abs(model.T - Tref).max()
        assert np.array_equal(model.Fsurf, fs)
    # the caller's T0 array is the model's T (reference aliasing)
    assert model.T is T_host


@pytest.mark.parametrize("nz", [40, 255])
def test_step_t_bitwise_vs_oracle(nz):
    rng = np.random.default_rng(5)
    n = 777
    z, ti, rhoc, T, _, _, _, Fg = _random_case(rng, n, nz)
    T = _smooth_if_fine(T, z)
    Ts = T[:, 0].copy()
    model = PccThermalModel1D(z, T.copy(), ti, rhoc, np.ones(n), Fg, np.zeros(n), Ts, bcond="T")
    Tref = T.copy()
    for step in range(3):
        X = rng.uniform(50, 350, n)
        fs = opcc.step_t(z, 3600.0, Ts, X, Tref, ti, rhoc, Fg)
        model.step(3600.0, X)
        Ts = X
        assert np.array_equal(model.T[:, 1:], Tref[:, 1:])
        assert np.array_equal(model.Fsurf, fs)


def test_golden_scenario_on_gpu():
    golden = np.load(GOLDEN / "pcc_conductionQ.npz")
    z = sc.grid(setgrid)
    w = z.size
    Qn, q = sc.fluxes(flux_noatm)
    model = PccThermalModel1D(z, np.full((1, w), 210.0), np.full(w, 120.0), np.full(w, 960000.0),
                              np.ones(1), np.full(1, 0.2), np.array([Qn]), np.array([210.0]))
    qd = torch.as_tensor(q, device="cuda")

    def step(i, dt):
        model.step(dt, qd[i:i + 1], check=False)

    prof, surf = sc.run(step, lambda: model.T_device[0].cpu().numpy(), q)
    model.check_errors()
    sc.check_against_golden(prof, surf, golden)


def test_errors_match_reference_messages_and_keep_state():
    rng = np.random.default_rng(1)
    z, ti, rhoc, T, Qprev, X, emiss, Fg = _random_case(rng, 64, 40)
    model = PccThermalModel1D(z, T.copy(), ti, rhoc, emiss, Fg, Qprev, T[:, 0].copy())
    before = model.T.copy()
    bad = X.copy()
    bad[3] = -1.0
    with pytest.raises(RuntimeError, match="trying to step with negative fluxes"):
        model.step(100.0, bad)
    bad[3] = np.nan
    with pytest.raises(RuntimeError, match="trying to step with nonfinite input fluxes"):
        model.step(100.0, bad)
    with pytest.raises(RuntimeError, match="input flux of wrong size"):
        model.step(100.0, X[:10])
    assert np.array_equal(model.T, before)
    assert model.current_time == 0
    with pytest.raises(ValueError, match="emissivity"):
        PccThermalModel1D(z, T.copy(), ti, rhoc, emiss + 1, Fg, Qprev, T[:, 0].copy())
    with pytest.raises(RuntimeError, match=r"z\[0\] is required to be zero"):
        PccThermalModel1D(z + 1, T.copy(), ti, rhoc, emiss, Fg, Qprev, T[:, 0].copy())


@pytest.mark.parametrize("nz", [40, 255])
def test_fp32_kernel_close_to_fp64(nz):
    """The FP32 kernel (one reciprocal per pivot) against the FP64 one; at
    nz = 255 the facets of a CTA are fewer (shared-memory budget)."""
    rng = np.random.default_rng(2)
    n = 2048
    z, ti, rhoc, T, Qprev, X, emiss, Fg = _random_case(rng, n, nz)
    T = _smooth_if_fine(T, z)
    m64 = PccThermalModel1D(z, T.copy(), ti, rhoc, emiss, Fg, Qprev, T[:, 0].copy())
    m32 = PccThermalModel1D(z, T.copy(), ti, rhoc, emiss, Fg, Qprev, T[:, 0].copy(),
                            dtype=np.float32)
    for _ in range(20):
        X = rng.uniform(0, 1200, n)
        m64.step(3000.0, X)
        m32.step(3000.0, X)
    # FP32 state: relative error of a few ulps per step, well under 1e-3 K
    assert np.max(np.abs(m32.T.astype(np.float64) - m64.T)) < 2e-3
