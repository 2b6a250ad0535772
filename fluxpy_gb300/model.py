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


def _as_columns(E):
    """(device tensor of shape (N, K), was-a-vector, was-on-the-host, numpy dtype)."""
    on_dev = isinstance(E, torch.Tensor)
    nd = E.ndim if on_dev else np.ndim(E)
    if nd not in (1, 2):
        raise Exception('E should be a vector or a 2D array')
    if on_dev:
        Ed = E
        dt = np.float64 if E.dtype == torch.float64 else np.float32
    else:
        En = np.asarray(E)
        dt = np.float64 if En.dtype != np.float32 else np.float32
        Ed = torch.as_tensor(En.astype(dt, copy=False), device=_lib.require_cuda())
    return Ed.reshape(Ed.shape[0], -1), nd == 1, not on_dev, dt


def _per_facet(v, like):
    """A scalar, or a per-facet array broadcast over the columns of `like`."""
    if np.isscalar(v) or np.ndim(v) == 0:
        return float(v)
    t = v.to(like.device, like.dtype) if isinstance(v, torch.Tensor) else \
        torch.as_tensor(np.asarray(v, dtype=np.float64), device=like.device).to(like.dtype)
    return t.reshape(-1, 1)


def _elementwise(v, like):
    """A scalar as a float; a per-facet array (numpy or tensor) as a tensor
    on ``like``'s device and dtype, for elementwise products with it (the
    reference multiplies numpy arrays, model.py:61-67, 223)."""
    if np.isscalar(v) or np.ndim(v) == 0:
        return float(v)
    if isinstance(v, torch.Tensor):
        return v.to(like.device, like.dtype)
    return torch.as_tensor(np.asarray(v), device=like.device).to(like.dtype)


def _tensor_core_operator(FF):
    from .compressed_form_factors import CompressedFormFactorMatrix
    return isinstance(FF, CompressedFormFactorMatrix)


def _split_product(FF, X):
    """F X for K columns (facet order) on the tensor cores with split-BF16
    operands (~17-bit, as the refinement residual; the FP32 CUDA-core
    product of 1,024 columns takes ~5x longer at 522k facets)."""
    N, K = X.shape
    Kp = -(-K // 8) * 8
    Xp = torch.zeros((N, Kp), dtype=torch.float32, device=X.device)
    Xp[:, :K] = FF.permute(X.to(torch.float32))
    Y = torch.empty_like(Xp)
    FF.split_product(Xp, Y)
    return FF.unpermute(Y[:, :K]).to(X.dtype)


def compute_steady_state_temp(FF, E, rho, emiss, Fsurf=0., clamp=True,
                              tol=np.finfo(np.float64).eps, method='jacobi'):
    """Steady-state surface temperature for one (E of shape (N,)) or K sun
    directions (E of shape (N, K); result (K, N)), src/flux/model.py:8-42.

    Every column goes through the same three device stages, all columns at
    once: the visible solve B = E + F (rho B) (one solve for the block, with
    the reference's single stopping test over all columns), one K-column
    product IR = F((1 - rho) B [+ Fsurf]) (with method 'batched-bf16' on
    the tensor cores, split-BF16 operands), and the infrared solve
    Q = IR + F Q.  The infrared stage solves each column to its own
    default tolerance (finfo.resolution * max|IR[:, k]|, as the reference's
    per-column solve does): the block is solved with every column scaled
    to unit maximum, and scaled back.  Then
    T = ((1 - rho) B + emiss Q [+ Fsurf]) / (emiss sigma))^(1/4).
    As in the reference, Fsurf enters (and the total is clamped) only for
    a single direction.  Host arrays in, host arrays out."""
    Ed, single, host, dt = _as_columns(E)
    apply = _device_operator(FF, Ed.device, dt)
    rho_c = _per_facet(rho, Ed)
    em_c = _per_facet(emiss, Ed)
    B = solve_radiosity(FF, Ed, rho, 'right', method)[0]
    if clamp:
        B = B.clamp_min(0)
    absorbed = (1 - rho_c) * B
    fs = _per_facet(Fsurf, Ed) if single else 0.0
    if method == 'batched-bf16' and not single and _tensor_core_operator(FF):
        IR = _split_product(FF, absorbed)
    else:
        IR = apply((absorbed + fs).contiguous())
    scale = IR.abs().amax(0)
    scale = torch.where(scale > 0, scale, torch.ones_like(scale))
    Q = solve_radiosity(FF, (IR / scale).contiguous(), 1, 'right', method)[0] * scale
    if clamp:
        Q = Q.clamp_min(0)
    total = absorbed + em_c * Q + fs
    if single and clamp:
        total = total.clamp_min(0)
    T = (total / (em_c * sigSB)) ** 0.25
    T = T[:, 0] if single else T.T.contiguous()
    return T.cpu().numpy() if host else T


def update_incoming_radiances(FF, E, rho, emiss, Qrefl, QIR, Tsurf, clamp=True):
    """Lagged reflected and infrared fluxes for one time step
    (model.py:44-69; eqs. 17-18 of the radiosity paper).  rho and emiss are
    scalars or per-facet arrays; a per-facet rho scales F (E + Qrefl)
    facet by facet.  (The reference's ``rho * FF @ (E + Qrefl)`` is
    ``(rho * FF) @ (E + Qrefl)``: the same for a scalar rho, but a
    vector-matrix product, and then a single number, for a per-facet
    array.)"""
    if isinstance(E, torch.Tensor):
        rho, emiss = _elementwise(rho, E), _elementwise(emiss, E)
        Qrefl_np1 = rho * _apply(FF, E + Qrefl)
        if clamp:
            Qrefl_np1 = torch.clamp_min(Qrefl_np1, 0)
        QIR_np1 = _apply(FF, emiss * sigSB * Tsurf**4 + (1 - emiss) * QIR)
        if clamp:
            QIR_np1 = torch.clamp_min(QIR_np1, 0)
        return Qrefl_np1, QIR_np1
    if np.isscalar(rho) or np.ndim(rho) == 0:
        Qrefl_np1 = rho * FF @ (E + Qrefl)
    else:
        Qrefl_np1 = np.asarray(rho) * (FF @ (E + Qrefl))
    if clamp:
        Qrefl_np1 = np.maximum(0, Qrefl_np1)
    QIR_np1 = FF @ (emiss * sigSB * Tsurf**4 + (1 - emiss) * QIR)
    if clamp:
        QIR_np1 = np.maximum(0, QIR_np1)
    return Qrefl_np1, QIR_np1


# Keyword inputs of ThermalModel, in the order they are checked: name, what
# it is (for the error message, model.py:133-172), and its shape as a
# function of (number of facets, number of grid nodes); None: not promoted.
_THERMAL_KWARGS = (
    ('z', 'skin depths', None),
    ('T0', 'initial temperature', lambda nf, nz: (nf, nz)),
    ('ti', 'thermal inertia', lambda nf, nz: (nz,)),
    ('rhoc', 'thermal conductivity', lambda nf, nz: (nz,)),
    ('emiss', 'emissivity', lambda nf, nz: (nf,)),
    ('Fgeotherm', 'geothermal flux', lambda nf, nz: (nf,)),
)


def _thermal_fields(kwargs, num_faces):
    """The conduction inputs of ThermalModel as arrays: a Python int or
    float fills the array, an ndarray must already have the shape."""
    out = {}
    nz = None
    for name, what, shape_of in _THERMAL_KWARGS:
        if name not in kwargs:
            raise ValueError(f'failed to pass {what} (keyword argument "{name}")')
        v = kwargs[name]
        if shape_of is None:
            assert not isinstance(v, int)
            out[name] = v
            nz = v.size
            continue
        shape = shape_of(num_faces, nz)
        if isinstance(v, (int, float)):
            v = np.full(shape, v, np.float64)
        elif not isinstance(v, np.ndarray):
            raise TypeError(f'bad type: {type(v)}')
        elif v.shape != shape:
            raise ValueError('invalid shape')
        out[name] = v
    return out


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
        self._t, self._D, self._F0, self._rho = t, D, F0, rho
        self._source_num_faces = D.shape[0] // t.shape[0]
        self._return_flux = return_flux
        fields = _thermal_fields(kwargs, self._shape_model.num_faces)
        z, T0, ti, rhoc = fields['z'], fields['T0'], fields['ti'], fields['rhoc']
        emiss, Fgeotherm = fields['emiss'], fields['Fgeotherm']

        # initial state from direct illumination only (model.py:165-171)
        E0 = self._insolation(0, device=False)
        Q0 = (1 - rho) * E0 + Fgeotherm
        Tsurf = (Q0 / (sigSB * emiss))**0.25
        self._pcc_thermal_model_1d = PccThermalModel1D(
            z, T0, ti, rhoc, emiss, Fgeotherm, Q0, Tsurf, bcond='Q')
        self._dev = _lib.require_cuda()
        self._Tsurf = torch.as_tensor(Tsurf, device=self._dev)
        self._rho_d = _elementwise(rho, self._Tsurf)
        self._emiss_d = self._pcc_thermal_model_1d.emiss_device
        self._iter_count = 0
        self._Qrefl = None
        self._QIR = None

    def _insolation(self, i, device=True):
        """Direct insolation at time point i: one sun direction per time
        point, or (source_num_faces > 1) that many source points averaged by
        the shape model.  The single-direction case runs as a one-column
        batch on the device."""
        s = self._source_num_faces
        if s == 1:
            if device:
                return self._shape_model.get_direct_irradiance_batch(
                    self._F0[i], self._D[i], out_dtype=torch.float64)[:, 0]
            return self._shape_model.get_direct_irradiance(self._F0[i], self._D[i])
        part = slice(i * s, (i + 1) * s)
        E = self._shape_model.get_direct_irradiance(self._F0[part], self._D[part])
        return torch.as_tensor(E, device=self._dev) if device else E

    def __iter__(self):
        return self

    def __next__(self):
        """One time step: E_i, the lagged fluxes from the previous step's
        state, the absorbed flux Q, one conduction step; returns the
        conduction profiles (and the fluxes with return_flux)."""
        self._iter_count += 1
        i = self._iter_count
        if i * self._source_num_faces >= self._D.shape[0]:
            raise StopIteration()
        E = self._insolation(i)
        dt = self._t[i] - self._t[i - 1]
        first = i == 1
        Qrefl, QIR = update_incoming_radiances(
            self._FF, E, self._rho_d, self._emiss_d,
            Qrefl=torch.zeros_like(E) if first else self._Qrefl,
            QIR=torch.zeros_like(E) if first else self._QIR, Tsurf=self._Tsurf)
        Q = (1 - self._rho_d) * (E + Qrefl) + self._emiss_d * QIR
        pcc = self._pcc_thermal_model_1d
        pcc.step(dt, Q)
        self._Qrefl, self._QIR = Qrefl, QIR
        self._Tsurf = pcc.T_device[:, 0].contiguous()
        if self._return_flux:
            return pcc.T, E.cpu().numpy(), Qrefl.cpu().numpy(), QIR.cpu().numpy()
        return pcc.T
