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


def test_thermal_model_checks_inputs_before_device_use():
    """ThermalModel's argument checks (model.py:110-172): sun positions,
    every required keyword in the reference's order, shapes and types."""
    from types import SimpleNamespace
    nf, nt = 6, 4
    sm = SimpleNamespace(num_faces=nf)
    t = np.linspace(0.0, 3600.0, nt)
    D = np.tile([0.0, 0.0, 1.0], (nt, 1))
    F0 = np.full(nt, 1365.0)
    z = np.array([0.0, 0.01, 0.03, 0.05])
    full = dict(z=z, T0=200.0, ti=100.0, rhoc=1e6, emiss=0.95, Fgeotherm=0.005)
    with pytest.raises(ValueError, match="N x 3 ndarray"):
        model.ThermalModel(None, t, D[:, :2], F0, 0.12, shape_model=sm, **full)
    with pytest.raises(ValueError, match="equal or multiple"):
        model.ThermalModel(None, t, D[:3], F0, 0.12, shape_model=sm, **full)
    names = ["z", "T0", "ti", "rhoc", "emiss", "Fgeotherm"]
    for i, name in enumerate(names):
        kw = {k: full[k] for k in names[:i]}
        with pytest.raises(ValueError, match=f'keyword argument "{name}"'):
            model.ThermalModel(None, t, D, F0, 0.12, shape_model=sm, **kw)
    with pytest.raises(ValueError, match="invalid shape"):
        model.ThermalModel(None, t, D, F0, 0.12, shape_model=sm,
                           **{**full, "emiss": np.full(nf + 1, 0.9)})
    with pytest.raises(ValueError, match="invalid shape"):
        model.ThermalModel(None, t, D, F0, 0.12, shape_model=sm,
                           **{**full, "T0": np.full((nf, z.size + 1), 200.0)})
    with pytest.raises(TypeError, match="bad type"):
        model.ThermalModel(None, t, D, F0, 0.12, shape_model=sm, **{**full, "ti": [100.0] * 4})
