"""Host logic of the thermal-model fluxes (no GPU): scalar and per-facet
albedo and emissivity, host arrays and tensors (the device product is
replaced by the same sparse product on the host)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch
from scipy.constants import Stefan_Boltzmann as sigSB

from fluxpy_gb300 import model


@pytest.fixture
def case(monkeypatch):
    rng = np.random.default_rng(0)
    n = 60
    FF = sp.random(n, n, density=0.2, random_state=1, format="csr") * 0.05
    monkeypatch.setattr(model, "_apply", lambda F, x: torch.as_tensor(F @ x.numpy()))
    E = rng.uniform(0, 1365, n)
    Qr, QIR, Ts = rng.uniform(0, 50, n), rng.uniform(0, 20, n), rng.uniform(150, 350, n)
    rho, emiss = rng.uniform(0.05, 0.3, n), rng.uniform(0.9, 1.0, n)
    return FF, E, Qr, QIR, Ts, rho, emiss


def test_scalar_albedo_is_the_reference_expression(case):
    FF, E, Qr, QIR, Ts, _, emiss = case
    a, b = model.update_incoming_radiances(FF, E, 0.12, 0.95, Qr, QIR, Ts)
    # model.py:61-67 as written
    assert np.array_equal(a, np.maximum(0, 0.12 * FF @ (E + Qr)))
    assert np.array_equal(b, np.maximum(0, FF @ (0.95 * sigSB * Ts**4 + (1 - 0.95) * QIR)))
    t = torch.as_tensor
    ad, bd = model.update_incoming_radiances(FF, t(E), 0.12, 0.95, t(Qr), t(QIR), t(Ts))
    assert np.allclose(ad.numpy(), a, rtol=1e-13, atol=0)
    assert np.allclose(bd.numpy(), b, rtol=1e-13, atol=0)


def test_per_facet_albedo_and_emissivity(case):
    FF, E, Qr, QIR, Ts, rho, emiss = case
    a_ref = np.maximum(0, rho * (FF @ (E + Qr)))
    b_ref = np.maximum(0, FF @ (emiss * sigSB * Ts**4 + (1 - emiss) * QIR))
    a, b = model.update_incoming_radiances(FF, E, rho, emiss, Qr, QIR, Ts)
    assert a.shape == E.shape
    assert np.allclose(a, a_ref, rtol=1e-14, atol=0) and np.allclose(b, b_ref, rtol=1e-14, atol=0)
    t = torch.as_tensor
    # tensors in: numpy or tensor albedo and emissivity
    for r, e in ((rho, emiss), (t(rho), t(emiss)), (list(rho), emiss)):
        ad, bd = model.update_incoming_radiances(FF, t(E), r, e, t(Qr), t(QIR), t(Ts))
        assert isinstance(ad, torch.Tensor) and ad.shape == E.shape
        assert np.allclose(ad.numpy(), a_ref, rtol=1e-13, atol=0)
        assert np.allclose(bd.numpy(), b_ref, rtol=1e-13, atol=0)


def test_elementwise_conversion():
    x = torch.zeros(4, dtype=torch.float64)
    assert model._elementwise(0.5, x) == 0.5 and isinstance(model._elementwise(np.float32(2), x), float)
    v = model._elementwise(np.arange(4, dtype=np.float32), x)
    assert v.dtype == torch.float64 and v.tolist() == [0.0, 1.0, 2.0, 3.0]
