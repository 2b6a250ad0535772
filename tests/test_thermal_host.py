"""CPU: PccThermalModel1D checks its inputs before it touches the device,
with the reference's exception types and messages (thermal.pyx:99-156);
valid inputs then need the GPU (no CPU fallback)."""
import numpy as np
import pytest
import torch

from fluxpy_gb300.thermal import PccThermalModel1D, setgrid


def _inputs(nf=5, nz=6):
    z = np.concatenate([[0.0], setgrid(nz, 1.1, 0.5)])
    return dict(z=z, T0=np.full((nf, z.size), 200.0), ti=np.full(z.size, 100.0),
                rhoc=np.full(z.size, 1e6), emiss=np.full(nf, 0.95), Fgeotherm=np.full(nf, 0.005),
                Q0=np.full(nf, 300.0), Tsurfprev=np.full(nf, 200.0))


CASES = [
    ("bcond", "X", ValueError, 'bcond should be "Q" or "T"'),
    ("emiss", np.full(5, 1.2), ValueError, r'emissivity values \("emiss"\) should be in range'),
    ("emiss", np.full(4, 0.9), ValueError, '"emiss" should be a 1D array'),
    ("z", None, RuntimeError, r"z\[0\] is required to be zero"),
    ("ti", -1.0, ValueError, r'thermal inertia \("ti"\) values should be positive'),
    ("ti", np.full(3, 100.0), ValueError, '"ti" should be a 1D array'),
    ("rhoc", 0.0, ValueError, r'volumetric heat capacity \("rhoc"\) values should be positive'),
    ("Fgeotherm", -1.0, ValueError, r'geothermal fluxes \("Fgeotherm"\) should be positive'),
    ("Tsurfprev", -1.0, ValueError, 'should be nonnegative'),
    ("Q0", -1.0, ValueError, r'initial irradiance \("Q0"\) should be nonnegative'),
    ("T0", -1.0, ValueError, r'initial temperature \("T0"\) should be nonnegative'),
]


@pytest.mark.parametrize("name,value,exc,msg", CASES)
def test_bad_inputs_raise_reference_messages(name, value, exc, msg):
    kw = _inputs()
    if name == "bcond":
        kw["bcond"] = value
    elif name == "z":
        kw["z"] = kw["z"] + 0.01
    elif np.ndim(value) == 0:
        kw[name] = np.full_like(kw[name], value)
    else:
        kw[name] = value
    with pytest.raises(exc, match=msg):
        PccThermalModel1D(**kw)


def test_grid_and_dtype_checks():
    kw = _inputs()
    kw.update(z=np.array([0.0, 0.1]), T0=np.full((5, 2), 200.0), ti=np.full(2, 100.0),
              rhoc=np.full(2, 1e6))
    with pytest.raises(ValueError, match="at least two layers"):
        PccThermalModel1D(**kw)
    with pytest.raises(ValueError, match="float64 or float32"):
        PccThermalModel1D(**_inputs(), dtype=np.float16)
    with pytest.raises(ValueError, match="bcond 'Q' only"):
        PccThermalModel1D(**_inputs(), bcond="T", dtype=np.float32)


def test_valid_inputs_need_the_gpu(monkeypatch):
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        PccThermalModel1D(**_inputs())
