"""GPU: ThermalModel and update_incoming_radiances (src/flux/model.py:44-234)
against a step-by-step restatement of the reference's iteration with the
oracle's conductionQ (oracle/pcc_oracle.c) and the exact form-factor matrix
applied by scipy, on the spherical crater of the reference fixtures."""
import numpy as np
import pytest
import torch
from scipy.constants import Stefan_Boltzmann as sigSB

from oracle import pcc as opcc
from tests.conftest import GOLDEN
from fluxpy_gb300 import shape as gshape
from fluxpy_gb300.form_factors import get_form_factor_matrix
from fluxpy_gb300.model import ThermalModel, update_incoming_radiances
from fluxpy_gb300.thermal import setgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def crater():
    ref = np.load(GOLDEN / "ffref.npz")
    sm = gshape.EmbreeTrimeshShapeModel(ref["crater_V"], ref["crater_F"])
    return sm, get_form_factor_matrix(sm)


def _sun(nt):
    elev = np.deg2rad(np.linspace(8.0, 40.0, nt))
    az = np.deg2rad(np.linspace(0.0, 75.0, nt))
    return np.column_stack([np.cos(elev) * np.cos(az), np.cos(elev) * np.sin(az), np.sin(elev)])


def test_update_incoming_radiances_host_and_device(crater):
    sm, FF = crater
    n = sm.num_faces
    rng = np.random.default_rng(1)
    E = rng.uniform(0, 1365, n)
    Qr, QIR, Ts = rng.uniform(0, 50, n), rng.uniform(0, 20, n), rng.uniform(150, 350, n)
    emiss = rng.uniform(0.9, 1.0, n)
    a, b = update_incoming_radiances(FF, E, 0.12, emiss, Qr, QIR, Ts)
    # model.py:61-67 in plain numpy / scipy
    a_ref = np.maximum(0, 0.12 * FF @ (E + Qr))
    b_ref = np.maximum(0, FF @ (emiss * sigSB * Ts**4 + (1 - emiss) * QIR))
    assert np.allclose(a, a_ref, rtol=1e-12, atol=0)
    assert np.allclose(b, b_ref, rtol=1e-12, atol=0)
    t = lambda x: torch.as_tensor(x, device="cuda")
    ad, bd = update_incoming_radiances(FF, t(E), 0.12, t(emiss), t(Qr), t(QIR), t(Ts))
    assert np.allclose(ad.cpu().numpy(), a_ref, rtol=1e-12, atol=1e-12 * abs(a_ref).max())
    assert np.allclose(bd.cpu().numpy(), b_ref, rtol=1e-12, atol=1e-12 * abs(b_ref).max())


def test_thermal_model_matches_restatement(crater):
    sm, FF = crater
    n = sm.num_faces
    nt = 7
    t = np.linspace(0.0, 6 * 3600.0, nt)
    D = _sun(nt)
    F0 = np.full(nt, 1365.0)
    rho, emiss, Fg, ti, rhoc, T0 = 0.12, 0.95, 0.005, 120.0, 960000.0, 210.0
    z = np.concatenate([[0.0], setgrid(20, 1.08, 0.5)])
    model = ThermalModel(FF, t, D, F0, rho, z=z, T0=T0, ti=ti, rhoc=rhoc, emiss=emiss,
                         Fgeotherm=Fg, shape_model=sm, return_flux=True)
    got = [(T.copy(), E.copy(), Qr.copy(), QIR.copy()) for T, E, Qr, QIR in model]
    assert len(got) == nt - 1
    # the reference's iteration (model.py:137-234), with the insolation of the
    # shape model (checked against the oracle's ray caster elsewhere)
    E_of = lambda i: sm.get_direct_irradiance(F0[i], D[i])
    em = np.full(n, emiss)
    Fgv = np.full(n, Fg)
    tiv, rhocv = np.full(z.size, ti), np.full(z.size, rhoc)
    Q0 = (1 - rho) * E_of(0) + Fgv
    Tsurf = (Q0 / (sigSB * em))**0.25
    T = np.full((n, z.size), T0)
    Qprev, Qrefl, QIR = Q0, np.zeros(n), np.zeros(n)
    for i in range(1, nt):
        E = E_of(i)
        Qrefl_n = np.maximum(0, rho * FF @ (E + Qrefl))
        QIR_n = np.maximum(0, FF @ (em * sigSB * Tsurf**4 + (1 - em) * QIR))
        Q = (1 - rho) * (E + Qrefl_n) + em * QIR_n
        opcc.step_q(z, t[i] - t[i - 1], Qprev, Q, T, tiv, rhocv, em, Fgv)
        Qprev, Qrefl, QIR, Tsurf = Q, Qrefl_n, QIR_n, T[:, 0].copy()
        Tg, Eg, Qrg, QIRg = got[i - 1]
        # the model evaluates the insolation with the batched device kernel,
        # get_direct_irradiance with numpy's dot product: equal to a few ulp
        assert np.allclose(Eg, E, rtol=1e-14, atol=1e-12)
        assert np.allclose(Qrg, Qrefl, rtol=1e-11, atol=1e-11 * max(abs(Qrefl).max(), 1.0))
        assert np.allclose(QIRg, QIR, rtol=1e-11, atol=1e-11 * max(abs(QIR).max(), 1.0))
        assert np.max(np.abs(Tg - T)) < 1e-8, (i, np.max(np.abs(Tg - T)))
    # errors as in the reference (model.py:111-115)
    with pytest.raises(ValueError):
        ThermalModel(FF, t, D[:, :2], F0, rho, z=z, T0=T0, ti=ti, rhoc=rhoc, emiss=emiss,
                     Fgeotherm=Fg, shape_model=sm)
    with pytest.raises(ValueError):
        ThermalModel(FF, t, D, F0, rho, T0=T0, ti=ti, rhoc=rhoc, emiss=emiss, Fgeotherm=Fg,
                     shape_model=sm)
