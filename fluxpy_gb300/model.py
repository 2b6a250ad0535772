"""Steady-state and time-dependent thermal models: drop-in for ``flux.model``.

``compute_steady_state_temp`` (src/flux/model.py:8-42),
``update_incoming_radiances`` (model.py:44-69) and ``ThermalModel``
(model.py:108-234) keep the reference's signatures and arithmetic; the
solves, products, insolation rays and the conduction step run on the GPU
(solve.py, compressed_form_factors.py, shape.py, thermal.py).
``ThermalModel`` keeps its state (fluxes, surface temperature, conduction
profiles) on the device between steps and hands back host arrays only when
iterated values are read.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.constants import Stefan_Boltzmann as sigSB

from . import _lib
from .solve import _device_operator, solve_radiosity
from .thermal import PccThermalModel1D


def _apply(FF, x):
    """FF @ x for host arrays (host result) or device tensors."""
    if isinstance(x, torch.Tensor):
        dt = np.float64 if x.dtype == torch.float64 else np.float32
        return _device_operator(FF, x.device, dt)(x)
    return FF @ x


def compute_steady_state_temp(FF, E, rho, emiss, Fsurf=0., clamp=True,
                              tol=np.finfo(np.float64).eps, method='jacobi'):
    """Steady-state surface temperature (model.py:8-42)."""
    if E.ndim == 1:
        B = solve_radiosity(FF, E, rho, 'right', method)[0]
        if clamp:
            B = np.maximum(0, B)
        IR = FF @ ((1 - rho) * B + Fsurf)
        Q = solve_radiosity(FF, IR, 1, 'right', method)[0]
        if clamp:
            Q = np.maximum(0, Q)
        tot = (1 - rho) * B + emiss * Q + Fsurf
        if clamp:
            tot = np.maximum(0, tot)
        return (tot / (emiss * sigSB))**0.25
    elif E.ndim == 2:
        B_arr = solve_radiosity(FF, E, rho, 'right', method)[0]
        if len(B_arr.shape) == 1:
            B_arr = B_arr[:, np.newaxis]
        T = []
        for B in B_arr.T:
            if clamp:
                B = np.maximum(0, B)
            IR = FF @ ((1 - rho) * B)
            Q = solve_radiosity(FF, IR, 1, 'right', method)[0]
            if clamp:
                Q = np.maximum(0, Q)
            T.append((((1 - rho) * B + emiss * Q) / (emiss * sigSB))**0.25)
        return np.array(T)
    else:
        raise Exception('E should be a vector or a 2D array')


def update_incoming_radiances(FF, E, rho, emiss, Qrefl, QIR, Tsurf, clamp=True):
    """Lagged reflected and infrared fluxes for one time step
    (model.py:44-69; eqs. 17-18 of the radiosity paper)."""
    if isinstance(E, torch.Tensor):
        Qrefl_np1 = rho * _apply(FF, E + Qrefl)
        if clamp:
            Qrefl_np1 = torch.clamp_min(Qrefl_np1, 0)
        QIR_np1 = _apply(FF, emiss * sigSB * Tsurf**4 + (1 - emiss) * QIR)
        if clamp:
            QIR_np1 = torch.clamp_min(QIR_np1, 0)
        return Qrefl_np1, QIR_np1
    Qrefl_np1 = rho * FF @ (E + Qrefl)
    if clamp:
        Qrefl_np1 = np.maximum(0, Qrefl_np1)
    QIR_np1 = FF @ (emiss * sigSB * Tsurf**4 + (1 - emiss) * QIR)
    if clamp:
        QIR_np1 = np.maximum(0, QIR_np1)
    return Qrefl_np1, QIR_np1


class ThermalModel:
    """Time-dependent thermal model (model.py:108-234): per step, direct
    insolation, lagged reflected/IR fluxes (two form-factor products) and a
    conduction step for every facet, all on the device."""

    def __init__(self, FF, t, D, F0, rho, method='1mvp', return_flux=False, **kwargs):
        if D.ndim != 2 or D.shape[1] != 3:
            raise ValueError('sun positions ("D") should be an N x 3 ndarray')
        if np.mod(D.shape[0], t.shape[0]) != 0:
            raise ValueError('number of sun positions ("D") should be equal or multiple of '
                             'number of time points ("t")')
        self._FF = FF
        self._shape_model = kwargs['shape_model'] if 'shape_model' in kwargs else FF.shape_model
        self._t = t
        self._D = D
        self._F0 = F0
        self._rho = rho
        self._source_num_faces = int(self._D.shape[0] / self._t.shape[0])
        self._return_flux = return_flux
        num_faces = self._shape_model.num_faces
        if 'z' not in kwargs:
            raise ValueError('failed to pass skin depths (keyword argument "z")')
        z = kwargs['z']

        def promote_to_array_if_necessary(value, shape, dtype=None):
            if isinstance(value, (int, float)):
                return np.full(shape, value, dtype)
            elif isinstance(value, np.ndarray):
                if value.shape != shape:
                    raise ValueError('invalid shape')
                return value
            else:
                raise TypeError(f'bad type: {type(value)}')

        assert not isinstance(z, int)
        if 'T0' not in kwargs:
            raise ValueError('failed to pass initial temperature (keyword argument "T0")')
        T0 = promote_to_array_if_necessary(kwargs['T0'], (num_faces, z.size), np.float64)
        if 'ti' not in kwargs:
            raise ValueError('failed to pass thermal inertia (keyword argument "ti")')
        ti = promote_to_array_if_necessary(kwargs['ti'], (z.size,), np.float64)
        if 'rhoc' not in kwargs:
            raise ValueError('failed to pass thermal conductivity (keyword argument "rhoc")')
        rhoc = promote_to_array_if_necessary(kwargs['rhoc'], (z.size,), np.float64)
        if 'emiss' not in kwargs:
            raise ValueError('failed to pass emissivity (keyword argument "emiss")')
        emiss = promote_to_array_if_necessary(kwargs['emiss'], (num_faces,), np.float64)
        if 'Fgeotherm' not in kwargs:
            raise ValueError('failed to pass geothermal flux (keyword argument "Fgeotherm")')
        Fgeotherm = promote_to_array_if_necessary(kwargs['Fgeotherm'], (num_faces,), np.float64)

        if self._source_num_faces == 1:
            E0 = self._shape_model.get_direct_irradiance(F0[0], D[0])
        else:
            E0 = self._shape_model.get_direct_irradiance(F0[:self._source_num_faces],
                                                         D[:self._source_num_faces])
        Q0 = (1 - rho) * E0 + Fgeotherm
        Tsurf = (Q0 / (sigSB * emiss))**0.25
        self._pcc_thermal_model_1d = PccThermalModel1D(
            z, T0, ti, rhoc, emiss, Fgeotherm, Q0, Tsurf, bcond='Q')
        dev = _lib.require_cuda()
        self._dev = dev
        self._Tsurf = torch.as_tensor(Tsurf, device=dev)
        self._emiss_d = self._pcc_thermal_model_1d.emiss_device
        self._iter_count = 0
        self._Qrefl = None
        self._QIR = None

    def __iter__(self):
        return self

    def __next__(self):
        self._iter_count += 1
        i = self._iter_count
        if (self._source_num_faces == 1) & (i == self._D.shape[0]):
            raise StopIteration()
        elif (self._source_num_faces > 1) & (self._source_num_faces * i == self._D.shape[0]):
            raise StopIteration()
        if self._source_num_faces == 1:
            f, d, delta_t = self._F0[i], self._D[i], self._t[i] - self._t[i - 1]
            E = self._shape_model.get_direct_irradiance_batch(
                f, d, out_dtype=torch.float64)[:, 0]
        else:
            f = self._F0[i * self._source_num_faces:(i + 1) * self._source_num_faces]
            d = self._D[i * self._source_num_faces:(i + 1) * self._source_num_faces, :]
            delta_t = self._t[i] - self._t[i - 1]
            E = torch.as_tensor(self._shape_model.get_direct_irradiance(f, d), device=self._dev)
        zero = torch.zeros_like(E)
        Qrefl_prev = zero if i == 1 else self._Qrefl
        QIR_prev = zero if i == 1 else self._QIR
        emiss = self._emiss_d
        Qrefl, QIR = update_incoming_radiances(self._FF, E, self._rho, emiss, Qrefl=Qrefl_prev,
                                               QIR=QIR_prev, Tsurf=self._Tsurf)
        Q = (1 - self._rho) * (E + Qrefl) + emiss * QIR
        self._pcc_thermal_model_1d.step(delta_t, Q)
        self._Qrefl = Qrefl
        self._QIR = QIR
        self._Tsurf = self._pcc_thermal_model_1d.T_device[:, 0].contiguous()
        if self._return_flux:
            return (self._pcc_thermal_model_1d.T, E.cpu().numpy(), Qrefl.cpu().numpy(),
                    QIR.cpu().numpy())
        return self._pcc_thermal_model_1d.T
