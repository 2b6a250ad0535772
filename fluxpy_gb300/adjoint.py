"""Hand-written adjoints of the radiosity solve and of the conduction step,
behind ``torch.autograd.Function`` (an addition: the reference computes no
derivatives).

* ``RadiositySolve`` / ``radiosity_solve(FF, E, rho)``: B with
  B = E + F (rho B) (the 'right' albedo placement of src/flux/solve.py:36-45),
  FP64 Jacobi on the device.  Backward: the transposed solve
  lam = gB + rho (F^T lam), then dL/dE = lam and dL/drho = B (F^T lam)
  (summed over columns); F^T is the compressed operator's transposed copy
  (``CompressedFormFactorMatrix.transposed``: the same kernels on the
  transposed blocks, deterministic) or a device CSR of F^T.  Many columns of
  a compressed FP32-stored operator are solved by iterative refinement:
  FP32 sweeps of all columns, FP64 residuals of all columns.
* ``ConductionStep`` / ``conduction_step(...)``: one conductionQ step
  (src/flux/pcc/conductionQ.c:10-186) with per-facet thermal inertia
  (``fgb_conduction_q_ti_f64``); backward: ``fgb_conduction_q_adjoint_f64``,
  the exact transposed Jacobian through the predictor-corrector passes.
* ``ThermalMisfit`` / ``thermal_misfit(...)``: the misfit of the coupled
  time-dependent model over S steps,
      B_n   = radiosity solve of the direct insolation E_n (all n at once)
      QIR_n = F (emiss sigma Ts_{n-1}^4 + (1 - emiss) QIR_{n-1})
              (the lagged infrared exchange of update_incoming_radiances,
              src/flux/model.py:44-69)
      Q_n   = (1 - rho) B_n + emiss QIR_n
      T_n   = conductionQ step (T_{n-1}; Q_{n-1}, Q_n; emiss, ti)
      L     = 0.5 sum_n sum_i (T_n[i, 0] - Tobs_n[i])^2,
  from Q_0 = (1 - rho) B_0 + Fgeotherm, Ts_0 = (Q_0 / (sigma emiss))^(1/4)
  and QIR_0 = 0 (the initial state of ThermalModel, model.py:165-171), and
  its gradient with respect to per-facet albedo, emissivity and thermal
  inertia by a hand-written reverse sweep: the forward pass keeps the state
  (profiles, fluxes) every ``checkpoint_every`` steps, each segment is
  recomputed from its checkpoint and swept backwards (conduction adjoint,
  F^T products of the infrared recursion), and one transposed radiosity
  solve per step turns the cotangents of B_n into the albedo gradient.

Everything runs in FP64 on the device; there is no CPU fallback.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse
import torch
from scipy.constants import Stefan_Boltzmann as SIGMA

from . import _lib
from .solve import NoConvergence, _DeviceCSR

F64 = torch.float64


# ------------------------------------------------------------ operators --
class _Ops:
    """y = F x and y = F^T x on FP64 device vectors in facet order (one
    column or K columns).  A compressed operator with FP32 storage applies
    K columns at once in FP64 arithmetic, its transpose through the
    transposed operator (``CompressedFormFactorMatrix.transposed``, same
    kernels, deterministic); ``batched`` tells the solves that they can
    refine with FP32 sweeps (``_refine``)."""

    def __init__(self, FF, dev):
        from .compressed_form_factors import CompressedFormFactorMatrix
        self.FF = FF
        self.batched = False
        if isinstance(FF, CompressedFormFactorMatrix):
            prec = "fp64" if FF._pool.dtype == torch.float64 else "fp32-fp64"
            self._prec = prec
            self.batched = prec == "fp32-fp64"

            def fwd(x):
                xp = FF.permute(x)
                if x.ndim == 1:
                    return FF.unpermute(FF.matvec_permuted(xp, prec))
                if self.batched:
                    return FF.unpermute(FF.matmat_permuted(xp.contiguous(), prec))
                return FF.unpermute(torch.stack([FF.matvec_permuted(xp[:, c].contiguous(), prec)
                                                 for c in range(xp.shape[1])], 1))

            def tr(y):
                yp = FF.permute(y)
                if y.ndim == 1:
                    return FF.unpermute(FF.rmatvec_permuted(yp, prec))
                if self.batched:
                    return FF.unpermute(FF.rmatmat_permuted(yp.contiguous(), prec))
                return FF.unpermute(torch.stack([FF.rmatvec_permuted(yp[:, c].contiguous(), prec)
                                                 for c in range(yp.shape[1])], 1))
            self.N = FF.num_faces
        elif scipy.sparse.issparse(FF) or isinstance(FF, np.ndarray):
            A = scipy.sparse.csr_matrix(FF)
            dF = _DeviceCSR(A, dev, np.float64)
            dT = _DeviceCSR(A.T.tocsr(), dev, np.float64)
            fwd, tr = dF.apply, dT.apply
            self.N = A.shape[0]
        else:
            raise TypeError(f"unsupported form factor operator: {type(FF)}")
        self._fwd, self._tr = fwd, tr

    def F(self, x):
        return self._fwd(x.contiguous())

    def FT(self, y):
        return self._tr(y.contiguous())


def _ops(FF, dev):
    cache = getattr(FF, "_fgb_adjoint_ops", None) if not isinstance(FF, np.ndarray) else None
    if cache is not None and cache[0] == dev:
        return cache[1]
    ops = _Ops(FF, dev)
    if not isinstance(FF, np.ndarray):
        try:
            FF._fgb_adjoint_ops = (dev, ops)
        except AttributeError:
            pass
    return ops


def _col(v, like):
    return v.reshape(-1, 1) if like.ndim == 2 else v


def _jacobi(apply, E, rho, tol, max_iter):
    """X = E + rho * apply(X) ... with rho applied on the side ``apply`` needs:
    the caller folds it in.  Stops when max|update| <= tol * max|E|."""
    X = E.clone()
    scale = float(E.abs().max().item()) if E.numel() else 0.0
    if scale == 0.0:
        return X, 0
    for it in range(1, max_iter + 1):
        X1 = apply(X, E)
        if float((X1 - X).abs().max().item()) <= tol * scale:
            return X1, it
        X = X1
    raise NoConvergence(f"Jacobi did not converge in {max_iter} iterations")


def _refine(ops, E, rho, tol, transpose, max_outer=30, sweep_tol=1e-7, max_sweeps=200):
    """Iterative refinement of the right-placement solve (transpose=False:
    B = E + F (rho B)) or of its transpose (lam = E + rho (F^T lam)) for K
    columns of a compressed FP32-stored operator: FP32 Jacobi sweeps of all
    columns for each correction (the FP32 K-column kernels), FP64 residuals
    of all columns (the FP32-stored operator in FP64 arithmetic) until
    max|E - (B - apply(B))| <= tol max|E|.  Works in cluster order."""
    FF = ops.FF
    Op = FF.transposed() if transpose else FF
    Ep = FF.permute(E).contiguous()
    rp = FF.permute(rho.expand(ops.N)).reshape(-1, 1).contiguous()
    rp32 = rp.to(torch.float32)
    scale = float(Ep.abs().max().item()) if Ep.numel() else 0.0
    if scale == 0.0:
        return torch.zeros_like(E)

    def ap64(X):
        if transpose:
            return rp * Op.matmat_permuted(X, "fp32-fp64")
        return Op.matmat_permuted((rp * X).contiguous(), "fp32-fp64")

    def ap32(X):
        if transpose:
            return rp32 * Op.matmat_permuted(X, "fp32")
        return Op.matmat_permuted((rp32 * X).contiguous(), "fp32")
    B = torch.zeros_like(Ep)
    R = Ep
    for _ in range(max_outer):
        R32 = R.to(torch.float32)
        thr = sweep_tol * float(R32.abs().max().item())
        D = R32.clone()
        for _ in range(max_sweeps):
            D1 = R32 + ap32(D)
            done = float((D1 - D).abs().max().item()) <= thr
            D = D1
            if done:
                break
        B = B + D.to(F64)
        R = Ep - (B - ap64(B))
        if float(R.abs().max().item()) <= tol * scale:
            return FF.unpermute(B)
    raise NoConvergence("refinement did not converge")


def solve_right(ops, E, rho, tol=1e-13, max_iter=10000):
    """B = E + F (rho B) for E (N,) or (N, K), FP64."""
    if ops.batched and E.ndim == 2:
        return _refine(ops, E, rho, tol, transpose=False)
    r = _col(rho, E)
    return _jacobi(lambda X, E_: E_ + ops.F(r * X), E, rho, tol, max_iter)[0]


def solve_right_T(ops, G, rho, tol=1e-13, max_iter=10000):
    """lam = G + rho (F^T lam): the transposed system of ``solve_right``."""
    if ops.batched and G.ndim == 2:
        return _refine(ops, G, rho, tol, transpose=True)
    r = _col(rho, G)
    return _jacobi(lambda X, G_: G_ + r * ops.FT(X), G, rho, tol, max_iter)[0]


# ------------------------------------------------------- radiosity solve --
class RadiositySolve(torch.autograd.Function):
    """B = (I - F diag(rho))^-1 E with its transposed-solve backward."""

    @staticmethod
    def forward(ctx, E, rho, FF, tol, max_iter):
        dev = E.device
        ops = _ops(FF, dev)
        E64 = E.detach().to(F64)
        rho64 = rho.detach().to(dev, F64).expand(ops.N).contiguous()
        B = solve_right(ops, E64, rho64, tol, max_iter)
        ctx.save_for_backward(B, rho64)
        ctx.ops, ctx.tol, ctx.max_iter = ops, tol, max_iter
        ctx.rho_shape = rho.shape
        return B.to(E.dtype)

    @staticmethod
    def backward(ctx, gB):
        B, rho64 = ctx.saved_tensors
        ops = ctx.ops
        lam = solve_right_T(ops, gB.to(F64).contiguous(), rho64, ctx.tol, ctx.max_iter)
        FTl = ops.FT(lam)
        grho = B * FTl
        if grho.ndim == 2:
            grho = grho.sum(1)
        if len(ctx.rho_shape) == 0 or ctx.rho_shape.numel() == 1:
            grho = grho.sum().reshape(ctx.rho_shape)
        return lam.to(gB.dtype), grho, None, None, None


def radiosity_solve(FF, E, rho, tol=1e-13, max_iter=10000):
    """Differentiable B = E + F (rho B) (device tensors; E (N,) or (N, K),
    rho a scalar tensor or (N,))."""
    _lib.require_cuda()
    if not isinstance(rho, torch.Tensor):
        rho = torch.as_tensor(rho, dtype=F64, device=E.device)
    return RadiositySolve.apply(E, rho, FF, tol, max_iter)


# ------------------------------------------------------- conduction step --
def _check_grid(z, T):
    if z.ndim != 1 or T.ndim != 2 or T.shape[1] != z.numel():
        raise ValueError('"T" should be a 2D array with T.shape[1] == z.size')
    if float(z[0]) != 0.0:
        raise RuntimeError("z[0] is required to be zero")


def _ti_full(ti, N, w):
    """(tensor, row stride) for the kernels: a per-layer profile (w,) is
    shared (stride 0); (N,) is uniform with depth per facet; (N, w) as is."""
    if ti.ndim == 1 and ti.numel() == w and N != w:
        return ti.contiguous(), 0
    if ti.ndim == 1 and ti.numel() == N:
        return ti.reshape(N, 1).expand(N, w).contiguous(), w
    if ti.ndim == 2 and ti.shape == (N, w):
        return ti.contiguous(), w
    raise ValueError('"ti" should have shape (nz+1,), (num_faces,) or (num_faces, nz+1)')


def _step(z, dt, Qn, Qnp1, T, ti, ld, rhoc, em, Fg, flags):
    N, w = T.shape
    out = torch.empty_like(T)
    _lib.call("fgb_conduction_q_ti_f64", N, w - 1, _lib.ptr(z), float(dt), _lib.ptr(Qn),
              _lib.ptr(Qnp1), _lib.ptr(T), _lib.ptr(out), _lib.ptr(ti), ld, _lib.ptr(rhoc),
              _lib.ptr(em), _lib.ptr(Fg), _lib.ptr(flags), _lib.stream_handle())
    return out


def _step_adjoint(z, dt, Qn, Qnp1, T, ti, ld, rhoc, em, Fg, gT, gem, gti, flags):
    N, w = T.shape
    gTin = torch.empty_like(T)
    gQn = torch.empty(N, dtype=F64, device=T.device)
    gQnp1 = torch.empty(N, dtype=F64, device=T.device)
    _lib.call("fgb_conduction_q_adjoint_f64", N, w - 1, _lib.ptr(z), float(dt), _lib.ptr(Qn),
              _lib.ptr(Qnp1), _lib.ptr(T), _lib.ptr(ti), ld, _lib.ptr(rhoc), _lib.ptr(em),
              _lib.ptr(Fg), _lib.ptr(gT.contiguous()), _lib.ptr(gTin), _lib.ptr(gQn),
              _lib.ptr(gQnp1), _lib.ptr(gem), _lib.ptr(gti), _lib.ptr(flags),
              _lib.stream_handle())
    return gTin, gQn, gQnp1


def _raise_flags(flags):
    f = int(flags.item())
    if f & _lib.FLAG_ZERO_PIVOT:
        raise RuntimeError("tridag failed")
    if f & _lib.FLAG_NONFINITE_OUT:
        raise RuntimeError("computed nonfinite temperatures while stepping")
    if f & _lib.FLAG_NEGATIVE_OUT:
        raise RuntimeError("computed negative temperatures while stepping")


class ConductionStep(torch.autograd.Function):
    """T_new = conductionQ(T; Qn, Qnp1, emiss, ti) for every facet."""

    @staticmethod
    def forward(ctx, T, Qn, Qnp1, emiss, ti, z, rhoc, dt, Fgeotherm):
        dev = T.device
        T64 = T.detach().to(F64).contiguous()
        N, w = T64.shape
        z64 = z.detach().to(dev, F64).contiguous()
        _check_grid(z64, T64)
        rhoc64 = rhoc.detach().to(dev, F64).contiguous()
        em = emiss.detach().to(dev, F64).contiguous()
        Fg = Fgeotherm.detach().to(dev, F64).contiguous()
        qn = Qn.detach().to(dev, F64).contiguous()
        qnp1 = Qnp1.detach().to(dev, F64).contiguous()
        tif, ld = _ti_full(ti.detach().to(dev, F64), N, w)
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
        out = _step(z64, dt, qn, qnp1, T64, tif, ld, rhoc64, em, Fg, flags)
        _raise_flags(flags)
        ctx.save_for_backward(T64, qn, qnp1, em, tif, z64, rhoc64, Fg)
        ctx.dt, ctx.ld, ctx.ti_shape = dt, ld, ti.shape
        return out.to(T.dtype)

    @staticmethod
    def backward(ctx, gT):
        T64, qn, qnp1, em, tif, z64, rhoc64, Fg = ctx.saved_tensors
        N, w = T64.shape
        gem = torch.zeros(N, dtype=F64, device=T64.device)
        gti = torch.zeros((N, w), dtype=F64, device=T64.device)
        flags = torch.zeros(1, dtype=torch.int32, device=T64.device)
        gTin, gQn, gQnp1 = _step_adjoint(z64, ctx.dt, qn, qnp1, T64, tif, ctx.ld, rhoc64, em, Fg,
                                         gT.to(F64), gem, gti, flags)
        shp = ctx.ti_shape
        if len(shp) == 1 and shp[0] == w and N != w:
            gti_out = gti.sum(0)
        elif len(shp) == 1:
            gti_out = gti.sum(1)
        else:
            gti_out = gti
        return gTin, gQn, gQnp1, gem, gti_out, None, None, None, None


def conduction_step(T, Qn, Qnp1, emiss, ti, z, rhoc, dt, Fgeotherm):
    """Differentiable conductionQ step on device tensors (FP64 arithmetic):
    T (N, nz+1), Qn, Qnp1, emiss, Fgeotherm (N,), ti (nz+1,), (N,) or
    (N, nz+1), z and rhoc (nz+1,)."""
    _lib.require_cuda()
    return ConductionStep.apply(T, Qn, Qnp1, emiss, ti, z, rhoc, dt, Fgeotherm)


# ------------------------------------------------------- coupled misfit --
class ThermalMisfit:
    """The coupled radiosity + conduction misfit (module docstring) for a
    fixed operator, insolation E (N, S+1), grid, initial profiles T0
    (N, nz+1), geothermal flux and observed surface temperatures Tobs
    (N, S); ``value_and_grad(rho, emiss, ti)`` runs the forward model and the
    hand-written reverse sweep."""

    def __init__(self, FF, E, z, rhoc, dt, T0, Fgeotherm, Tobs, checkpoint_every=25,
                 tol=1e-13, max_iter=10000):
        dev = _lib.require_cuda()
        self.dev = dev
        self.ops = _ops(FF, dev)

        def d(x):
            return torch.as_tensor(x, device=dev).to(F64).contiguous() \
                if not isinstance(x, torch.Tensor) else x.detach().to(dev, F64).contiguous()
        self.E = d(E)
        self.z = d(z)
        self.rhoc = d(rhoc)
        self.T0 = d(T0)
        self.Fg = d(Fgeotherm)
        self.Tobs = d(Tobs)
        self.dt = float(dt)
        N, S1 = self.E.shape
        if N != self.ops.N:
            raise ValueError("E should have one row per facet")
        if S1 < 2:
            raise ValueError("E should hold the insolation at steps 0..S, S >= 1")
        if self.Tobs.shape != (N, S1 - 1):
            raise ValueError('"Tobs" should have shape (num_faces, S)')
        _check_grid(self.z, self.T0)
        if self.T0.shape[0] != N or self.Fg.shape != (N,):
            raise ValueError("T0 / Fgeotherm do not match the number of facets")
        if checkpoint_every < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.N, self.S = N, S1 - 1
        self.C = int(checkpoint_every)
        self.tol, self.max_iter = tol, max_iter

    # forward state after step n: (T_n, Q_n, Ts_n, QIR_n)
    def _initial(self, B, rho, em):
        Q0 = (1 - rho) * B[:, 0] + self.Fg
        Ts0 = (Q0 / (SIGMA * em))**0.25
        return (self.T0.clone(), Q0, Ts0, torch.zeros_like(Q0))

    def _advance(self, n, state, B, rho, em, tif, ld, flags, record=None):
        T, Q, Ts, QIR = state
        QIRn = self.ops.F(em * SIGMA * Ts**4 + (1 - em) * QIR)
        Qn1 = (1 - rho) * B[:, n] + em * QIRn
        Tn = _step(self.z, self.dt, Q, Qn1, T, tif, ld, self.rhoc, em, self.Fg, flags)
        Tsn = Tn[:, 0].contiguous()
        if record is not None:
            record.append((T, Q, Qn1, Ts, QIR, QIRn, Tsn))
        return (Tn, Qn1, Tsn, QIRn)

    def _params(self, rho, emiss, ti):
        def d(x):
            return x.detach().to(self.dev, F64).contiguous() if isinstance(x, torch.Tensor) \
                else torch.as_tensor(np.asarray(x, np.float64), device=self.dev)
        rho, em, ti = d(rho), d(emiss), d(ti)
        N, w = self.N, self.z.numel()
        if rho.shape != (N,) or em.shape != (N,):
            raise ValueError('"rho" and "emiss" should have one value per facet')
        if ti.shape not in ((N,), (N, w)):
            raise ValueError('"ti" should have shape (num_faces,) or (num_faces, nz+1)')
        tif, ld = _ti_full(ti, N, w)
        return rho, em, ti, tif, ld

    def surface_temperatures(self, rho, emiss, ti):
        """Forward model only: Ts_n for n = 1..S as an (N, S) device tensor
        (e.g. synthetic observations from known fields)."""
        rho, em, ti, tif, ld = self._params(rho, emiss, ti)
        flags = torch.zeros(1, dtype=torch.int32, device=self.dev)
        B = solve_right(self.ops, self.E, rho, self.tol, self.max_iter)
        st = self._initial(B, rho, em)
        out = torch.empty((self.N, self.S), dtype=F64, device=self.dev)
        for n in range(1, self.S + 1):
            st = self._advance(n, st, B, rho, em, tif, ld, flags)
            out[:, n - 1] = st[2]
        _raise_flags(flags)
        return out

    def value(self, rho, emiss, ti):
        rho, em, ti, tif, ld = self._params(rho, emiss, ti)
        flags = torch.zeros(1, dtype=torch.int32, device=self.dev)
        B = solve_right(self.ops, self.E, rho, self.tol, self.max_iter)
        st = self._initial(B, rho, em)
        L = torch.zeros((), dtype=F64, device=self.dev)
        for n in range(1, self.S + 1):
            st = self._advance(n, st, B, rho, em, tif, ld, flags)
            L = L + 0.5 * torch.sum((st[2] - self.Tobs[:, n - 1])**2)
        _raise_flags(flags)
        return L

    def value_and_grad(self, rho, emiss, ti):
        """(L, dL/drho, dL/demiss, dL/dti) as FP64 device tensors; dL/dti has
        the shape of ``ti``."""
        rho, em, ti, tif, ld = self._params(rho, emiss, ti)
        N, S, C = self.N, self.S, self.C
        w = self.z.numel()
        dev = self.dev
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
        B = solve_right(self.ops, self.E, rho, self.tol, self.max_iter)
        # forward: misfit and checkpoints (state after steps 0, C, 2C, ...)
        st = self._initial(B, rho, em)
        ckpt = {0: st}
        L = torch.zeros((), dtype=F64, device=dev)
        for n in range(1, S + 1):
            st = self._advance(n, st, B, rho, em, tif, ld, flags)
            L = L + 0.5 * torch.sum((st[2] - self.Tobs[:, n - 1])**2)
            if n % C == 0 and n < S:
                ckpt[n] = st
        _raise_flags(flags)
        Ts0 = ckpt[0][2]
        Q0 = ckpt[0][1]
        # reverse sweep, one checkpointed segment at a time
        grho = torch.zeros(N, dtype=F64, device=dev)
        gem = torch.zeros(N, dtype=F64, device=dev)
        gti = torch.zeros((N, w), dtype=F64, device=dev)
        gB = torch.zeros_like(B)
        gT = torch.zeros((N, w), dtype=F64, device=dev)
        gQ_next = torch.zeros(N, dtype=F64, device=dev)
        gQIR_next = torch.zeros(N, dtype=F64, device=dev)
        starts = sorted(ckpt)
        for s0 in reversed(starts):
            s1 = min(s0 + C, S)
            rec = []
            st = ckpt[s0]
            for n in range(s0 + 1, s1 + 1):
                st = self._advance(n, st, B, rho, em, tif, ld, flags, record=rec)
            for n in range(s1, s0, -1):
                Tprev, Qprev, Qn1, Tsprev, QIRprev, QIRn, Tsn = rec[n - s0 - 1]
                gT[:, 0] += Tsn - self.Tobs[:, n - 1]
                gTp, gQa, gQb = _step_adjoint(self.z, self.dt, Qprev, Qn1, Tprev, tif, ld,
                                              self.rhoc, em, self.Fg, gT, gem, gti, flags)
                gQn = gQb + gQ_next
                gQ_next = gQa
                gB[:, n] += (1 - rho) * gQn
                grho -= B[:, n] * gQn
                gem += QIRn * gQn
                gQIR = em * gQn + gQIR_next
                gu = self.ops.FT(gQIR)
                gem += (SIGMA * Tsprev**4 - QIRprev) * gu
                gTs = 4 * em * SIGMA * Tsprev**3 * gu
                gQIR_next = (1 - em) * gu
                gT = gTp
                if n > 1:
                    gT[:, 0] += gTs
                else:
                    gQ_next = gQ_next + gTs * 0.25 * Ts0 / Q0
                    gem += gTs * (-0.25) * Ts0 / em
            del rec
        gB[:, 0] += (1 - rho) * gQ_next
        grho -= B[:, 0] * gQ_next
        lam = solve_right_T(self.ops, gB, rho, self.tol, self.max_iter)
        grho += torch.sum(B * self.ops.FT(lam), dim=1)
        _raise_flags(flags)
        gti_out = gti.sum(1) if ti.ndim == 1 else gti
        return L, grho, gem, gti_out


class _MisfitFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, emiss, ti, model):
        if any(ctx.needs_input_grad[:3]):
            L, gr, ge, gt = model.value_and_grad(rho, emiss, ti)
            ctx.save_for_backward(gr, ge, gt)
        else:
            L = model.value(rho, emiss, ti)
        return L

    @staticmethod
    def backward(ctx, gL):
        gr, ge, gt = ctx.saved_tensors
        return gL * gr, gL * ge, gL * gt, None


def thermal_misfit(model: ThermalMisfit, rho, emiss, ti):
    """L(rho, emiss, ti) of a ``ThermalMisfit`` as a differentiable scalar:
    ``thermal_misfit(m, rho, emiss, ti).backward()`` fills the three fields'
    ``.grad`` from the hand-written reverse sweep."""
    return _MisfitFn.apply(rho, emiss, ti, model)
