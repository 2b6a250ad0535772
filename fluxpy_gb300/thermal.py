"""Per-facet 1-D conduction on the GPU: drop-in for ``flux.thermal``.

``PccThermalModel1D`` keeps the reference constructor, properties, checks and
messages (src/flux/thermal.pyx:13-299); ``step`` advances every facet with
one launch of the batched Crank-Nicolson kernel (libfluxgb
``fgb_conduction_q_f64`` / ``fgb_conduction_t_f64``) instead of the serial
C loop over ``conductionQ`` (thermal.pyx:249-261).

State lives on the device.  The reference mutates the caller's ``T0`` array
in place (thermal.pyx:152 keeps a memoryview of it); here the caller's array
is refreshed from the device whenever ``.T`` is read, and ``.T_device`` gives
the device tensor without a copy.  A step whose input is rejected leaves the
state untouched, as the reference raises before calling ``conductionQ``.
"""
from __future__ import annotations

from math import acos, cos, pi, sin, sqrt

import numpy as np
import torch

from . import _lib


def _as_f64(x, name):
    if isinstance(x, torch.Tensor):
        return x.detach().to("cpu", torch.float64).numpy()
    a = np.asarray(x)
    return a


class PccThermalModel1D:
    """Bundle of 1-D thermal models, one per facet (thermal.pyx:13).

    Parameters mirror ``PccThermalModel1D.__cinit__`` (thermal.pyx:89-156):
    z (nz+1,) with z[0] == 0, T0 (num_faces, nz+1), ti and rhoc (nz+1,),
    emiss, Fgeotherm, Q0, Tsurfprev (num_faces,), bcond 'Q' or 'T'.
    ``dtype=np.float32`` selects the FP32 kernel (bcond 'Q' only).
    """

    def __init__(self, z, T0, ti, rhoc, emiss, Fgeotherm, Q0, Tsurfprev, bcond="Q",
                 dtype=np.float64):
        if bcond not in {"Q", "T"}:
            raise ValueError('bcond should be "Q" or "T"')
        self._bcond = bcond
        self._host_T = T0 if isinstance(T0, np.ndarray) else None
        T0n = _as_f64(T0, "T0")
        z = _as_f64(z, "z")
        ti = _as_f64(ti, "ti")
        rhoc = _as_f64(rhoc, "rhoc")
        emiss = _as_f64(emiss, "emiss")
        Fgeotherm = _as_f64(Fgeotherm, "Fgeotherm")
        Q0 = _as_f64(Q0, "Q0")
        Tsurfprev = _as_f64(Tsurfprev, "Tsurfprev")

        self._num_faces = T0n.shape[0]
        self._num_layers = z.size
        self._num_layers_interior = self._num_layers - 1
        self._current_time = 0

        if not all(0 <= _ <= 1 for _ in emiss):
            raise ValueError('emissivity values ("emiss") should be in range [0, 1]')
        if emiss.ndim != 1 or emiss.size != self.num_faces:
            raise ValueError('"emiss" should be a 1D array with length == T0.shape[0]')
        if z[0] != 0:
            raise RuntimeError("z[0] is required to be zero")
        if (ti <= 0.0).any():
            raise ValueError('thermal inertia ("ti") values should be positive')
        if ti.ndim != 1 or ti.size != self.num_layers:
            raise ValueError('"ti" should be a 1D array with length == z.size')
        if (rhoc <= 0).any():
            raise ValueError('volumetric heat capacity ("rhoc") values should be positive')
        if rhoc.ndim != 1 or rhoc.size != self.num_layers:
            raise ValueError('"rhoc" should be a 1D array with length == z.size')
        if (Fgeotherm < 0).any():
            raise ValueError('geothermal fluxes ("Fgeotherm") should be positive')
        if Fgeotherm.ndim != 1 or Fgeotherm.size != self.num_faces:
            raise ValueError('"Fgeotherm" should be a 1D array with length == T0.shape[0]')
        if (Tsurfprev < 0).any():
            raise ValueError('surface temperatures ("Tsurfprev") should be nonnegative')
        if Tsurfprev.ndim != 1 or Tsurfprev.size != self.num_faces:
            raise ValueError('"Tsurfprev" should be a 1D array with length == T0.shape[0]')
        if (Q0 < 0).any():
            raise ValueError('initial irradiance ("Q0") should be nonnegative')
        if Q0.ndim != 1 or Q0.size != self.num_faces:
            raise ValueError('"Q0" should be a 1D array with length == T0.shape[0]')
        if (T0n < 0).any():
            raise ValueError('initial temperature ("T0") should be nonnegative')
        if T0n.ndim != 2 or T0n.shape[1] != self.num_layers:
            raise ValueError('"T0" should be a 2D array with T0.shape[1] == z.size')
        if self._num_layers_interior < 2:
            raise ValueError("need at least two layers below the surface")

        self._dtype = np.dtype(dtype)
        if self._dtype not in (np.float64, np.float32):
            raise ValueError("dtype must be float64 or float32")
        if self._dtype == np.float32 and bcond != "Q":
            raise ValueError("the FP32 kernel implements bcond 'Q' only")
        tdt = torch.float64 if self._dtype == np.float64 else torch.float32
        dev = _lib.require_cuda()
        _lib.lib()
        self._device = dev
        self._tdt = tdt

        def d(a):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=tdt).to(dev)

        self._z = d(z)
        self._ti = d(ti)
        self._rhoc = d(rhoc)
        self._emiss = d(emiss)
        self._Fgeotherm = d(Fgeotherm)
        self._Qprev = d(Q0)
        self._Tsurfprev = d(Tsurfprev)
        self._Fsurf = torch.full((self._num_faces,), float("nan"), dtype=tdt, device=dev)
        self._T = d(T0n)
        self._T_next = torch.empty_like(self._T)
        self._flags = torch.zeros(1, dtype=torch.int32, device=dev)

    # -- properties (thermal.pyx:33-87) ---------------------------------
    @property
    def num_layers(self):
        return self._num_layers

    @property
    def num_faces(self):
        return self._num_faces

    @property
    def num_layers_interior(self):
        return self._num_layers_interior

    @property
    def current_time(self):
        return self._current_time

    @property
    def emiss(self):
        return self._emiss.cpu().numpy()

    @property
    def z(self):
        return self._z.cpu().numpy()

    @property
    def ti(self):
        return self._ti.cpu().numpy()

    @property
    def rhoc(self):
        return self._rhoc.cpu().numpy()

    @property
    def Fgeotherm(self):
        return self._Fgeotherm.cpu().numpy()

    @property
    def Qprev(self):
        return self._Qprev.cpu().numpy()

    @property
    def Fsurf(self):
        return self._Fsurf.cpu().numpy()

    @property
    def Tsurfprev(self):
        return self._Tsurfprev.cpu().numpy()

    @property
    def bcond(self):
        return self._bcond

    @property
    def T(self):
        """Temperature profiles (num_faces, nz+1), refreshed from the device.

        If the model was built from a float64 numpy ``T0``, that same array is
        updated and returned (the reference's aliasing of ``T0``)."""
        host = self._T.cpu().numpy()
        if (self._host_T is not None and self._host_T.dtype == host.dtype
                and self._host_T.shape == host.shape and self._host_T.flags.writeable):
            self._host_T[...] = host
            return self._host_T
        return host

    @property
    def T_device(self) -> torch.Tensor:
        return self._T

    @property
    def emiss_device(self) -> torch.Tensor:
        return self._emiss

    # -- stepping (thermal.pyx:236-299) ---------------------------------
    def _input(self, X):
        if isinstance(X, torch.Tensor):
            t = X.detach()
            if t.device != self._device or t.dtype != self._tdt:
                t = t.to(self._device, self._tdt)
            return t.contiguous()
        a = np.asarray(X)
        return torch.as_tensor(np.ascontiguousarray(a), dtype=self._tdt).to(self._device)

    def step(self, dt, X, check=True):
        """Advance every facet by ``dt`` with surface flux (bcond 'Q') or
        surface temperature (bcond 'T') ``X`` of length num_faces.

        With ``check=False`` the device flags are not read back, so the step
        is fully asynchronous; errors are then reported by the next checked
        step or by ``check_errors()``."""
        X_is_arr = isinstance(X, (np.ndarray, torch.Tensor))
        ndim = X.ndim if X_is_arr else np.ndim(X)
        size = (X.numel() if isinstance(X, torch.Tensor) else np.size(X))
        if self._bcond == "Q":
            if ndim != 1 or size != self._num_faces:
                raise RuntimeError(f"input flux of wrong size: X.size == {size}")
        elif self._bcond == "T":
            if ndim != 1 or size != self._num_faces:
                raise RuntimeError(f"input flux of wrong size: X.size == {size}")
        else:
            raise RuntimeError(f'got unexpected BC mode: "{self.bcond}"')
        Xd = self._input(X)
        stream = _lib.stream_handle()
        self._flags.zero_()
        nz = self._num_layers_interior
        if self._bcond == "Q":
            fn = "fgb_conduction_q_f64" if self._dtype == np.float64 else "fgb_conduction_q_f32"
            _lib.call(fn, self._num_faces, nz, _lib.ptr(self._z), float(dt),
                      _lib.ptr(self._Qprev), _lib.ptr(Xd), _lib.ptr(self._T),
                      _lib.ptr(self._T_next), _lib.ptr(self._ti), _lib.ptr(self._rhoc),
                      _lib.ptr(self._emiss), _lib.ptr(self._Fgeotherm), _lib.ptr(self._Fsurf),
                      _lib.ptr(self._flags), stream)
        else:
            _lib.call("fgb_conduction_t_f64", self._num_faces, nz, _lib.ptr(self._z),
                      float(dt), _lib.ptr(self._Tsurfprev), _lib.ptr(Xd), _lib.ptr(self._T),
                      _lib.ptr(self._T_next), _lib.ptr(self._ti), _lib.ptr(self._rhoc),
                      _lib.ptr(self._Fgeotherm), _lib.ptr(self._Fsurf), _lib.ptr(self._flags),
                      stream)
        if check:
            flags = int(self._flags.item())
            what = "fluxes" if self._bcond == "Q" else "temps"
            if flags & _lib.FLAG_NONFINITE_IN:
                raise RuntimeError(f"trying to step with nonfinite input {what}"
                                   if self._bcond == "T" else
                                   "trying to step with nonfinite input fluxes")
            if flags & _lib.FLAG_NEGATIVE_IN:
                raise RuntimeError("trying to step with negative fluxes" if self._bcond == "Q"
                                   else "trying to step with negative input temps")
        self._T, self._T_next = self._T_next, self._T
        if self._bcond == "Q":
            self._Qprev = Xd if Xd is not X else Xd.clone()
        else:
            self._Tsurfprev = Xd if Xd is not X else Xd.clone()
        if check:
            if flags & _lib.FLAG_ZERO_PIVOT:
                raise RuntimeError("tridag failed")
            if flags & _lib.FLAG_NONFINITE_OUT:
                raise RuntimeError("computed nonfinite temperatures while stepping")
            if flags & _lib.FLAG_NEGATIVE_OUT:
                raise RuntimeError("computed negative temperatures while stepping")
        self._current_time += dt

    def check_errors(self):
        flags = int(self._flags.item())
        if flags & (_lib.FLAG_NONFINITE_IN | _lib.FLAG_NONFINITE_OUT):
            raise RuntimeError("computed nonfinite temperatures while stepping")
        if flags & (_lib.FLAG_NEGATIVE_IN | _lib.FLAG_NEGATIVE_OUT):
            raise RuntimeError("computed negative temperatures while stepping")
        if flags & _lib.FLAG_ZERO_PIVOT:
            raise RuntimeError("tridag failed")


def setgrid(nz, zfac, zmax):
    """Regular or geometrically spaced 1-D grid (thermal.pyx:301-326): returns
    nz depths without the leading surface point, z[-1] == zmax."""
    z = [0]
    if zfac > 1.:
        dz = zmax / (3. + 2. * zfac * (zfac**(nz - 2) - 1.) / (zfac - 1.))
        z.append(dz)
        z.append(3 * z[1])
        for i in range(nz + 1)[3:]:
            z.append((1 + zfac) * z[i - 1] - zfac * z[i - 2])
    else:
        dz = zmax / nz
        z.extend([(i - 0.5) * dz for i in range(nz + 1)[1:]])
    return np.array(z)[1:]


def analytT_(z, T0, rhoc, ti, P, dt):
    """Analytic response to a sinusoidal surface temperature in a half-space
    (thermal.pyx:329-347)."""
    Ta = 30.
    delta = ti / rhoc * np.sqrt(P / np.pi)
    w = 2 * np.pi / P
    T = []
    for t in np.arange(0, P, dt)[:]:
        T.append(T0 + Ta * np.exp(-z / delta) * np.sin(z / delta - w * t))
    return np.vstack(T)


def flux_noatm(R, decl, latitude, HA, SlopeAngle, azFac):
    """Solar flux on a (sloped) surface without atmosphere (thermal.pyx:349-396)."""
    So = 1365.
    c1 = cos(latitude) * cos(decl)
    s1 = sin(latitude) * sin(decl)
    sinbeta = c1 * cos(HA) + s1
    cosbeta = sqrt(1 - sinbeta**2)
    buf = (sin(decl) - sin(latitude) * sinbeta) / (cos(latitude) * cosbeta)
    if buf > +1.:
        buf = +1.0
    if buf < -1.:
        buf = -1.0
    azSun = acos(buf)
    if sin(HA) >= 0:
        azSun = 2 * pi - azSun
    sintheta = cos(SlopeAngle) * sinbeta - sin(SlopeAngle) * cosbeta * cos(azSun - azFac)
    if cosbeta == 0.:
        sintheta = cos(SlopeAngle) * sinbeta
    if sintheta < 0.:
        sintheta = 0.
    if sinbeta < 0.:
        sintheta = 0.
    return sintheta * So / (R**2)
