"""Uneven batches of independent meshes: one launch per kernel for all of them.

``BlockDiagonalOperator`` merges the compressed operators of M independent
meshes (``CompressedFormFactorMatrix``, each in its own cluster order) into
one block-diagonal operator F = diag(F_1, ..., F_M) in one panel layout: mesh
i's rows start at R_i = sum_{j<i} ceil64(N_j) of a merged cluster order, so
no 64-row tile mixes meshes, and its groups, work items, tiles, Z rows, panel
rows and phase-A panel are appended with offsets (phase-B sources map
Z rows -> Z rows + Z_i, X rows -> the merged X rows).  One product of the
merged operator is then one phase-A and one phase-B launch over all meshes,
whatever their sizes (libfluxgb ``fgb_matvec_f32``, the same kernels and the
same per-tile order of sums as a single mesh's product).

``MultiMeshThermalModel`` runs the time-dependent model of ``ThermalModel``
(src/flux/model.py:108-234: per step, the lagged reflected and infrared
fluxes of update_incoming_radiances, model.py:44-69, and one conductionQ
step, src/flux/pcc/conductionQ.c:10-186) for all meshes at once in FP32:
all state (profiles, fluxes) lives in the merged cluster order; the
insolation of every mesh and step is computed up front by the batched ray
kernel; one step is two merged products, a few elementwise kernels and one
conduction launch over every facet of every mesh.  With ``use_graph`` the
steps are captured once in a CUDA graph (two steps per graph: the profile
and flux buffers alternate) and replayed, removing the per-launch host cost.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch
from scipy.constants import Stefan_Boltzmann as SIGMA

from . import _lib
from .compressed_form_factors import TILE_ROWS, fgb_op_desc


def _ceil64(n):
    return (n + TILE_ROWS - 1) // TILE_ROWS * TILE_ROWS


class BlockDiagonalOperator:
    """diag(F_1, ..., F_M) of independent meshes' compressed operators as one
    panel operator (module docstring).  Vectors are in the merged cluster
    order (length ``num_rows``, a multiple of 64; rows past a mesh's facets
    are padding: they read as zero and are written as zero)."""

    def __init__(self, ops, precision="fp32"):
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        if not ops:
            raise ValueError("need at least one operator")
        dev = ops[0]._perm_d.device
        self.precision = precision
        self.num_meshes = len(ops)
        self.mesh_faces = [int(op.num_faces) for op in ops]
        self.row0 = np.zeros(len(ops) + 1, np.int64)
        np.cumsum([_ceil64(n) for n in self.mesh_faces], out=self.row0[1:])
        self.num_rows = int(self.row0[-1])
        self.num_faces = int(sum(self.mesh_faces))
        nz = [int(op._num_zrows) for op in ops]
        z0 = np.concatenate([[0], np.cumsum(nz)]).astype(np.int64)
        self.num_zrows = int(z0[-1])
        if self.num_zrows + self.num_rows >= 2**31:
            raise OverflowError("merged operator too large for 32-bit panel sources")
        cat = {k: [] for k in ("g_c0", "g_n", "g_kz", "g_ldv", "g_voff", "g_z0", "a_grp", "a_j0",
                               "a_j1", "a_excl", "a_woff", "t_p0", "src")}
        panels, vpanels = [], []
        G = W = P = V = 0
        max_gt = 1
        needs_zero = False
        for i, op in enumerate(ops):
            d = op._dev
            ng = int(op.stats["groups"])
            ni = int(op._desc.num_items)
            nt = int(op._desc.num_tiles)
            rows = int(op._panel_rows)
            R = int(self.row0[i])
            cat["g_c0"].append(d["g_c0"][:ng].to(torch.int64) + R)
            for k in ("g_n", "g_kz", "g_ldv"):
                cat[k].append(d[k][:ng].to(torch.int64))
            cat["g_voff"].append(d["g_voff"][:ng] + V)
            cat["g_z0"].append(d["g_z0"][:ng] + int(z0[i]))
            cat["a_grp"].append(d["a_grp"][:ni].to(torch.int64) + G)
            cat["a_j0"].append(d["a_j0"][:ni].to(torch.int64))
            cat["a_j1"].append(d["a_j1"][:ni].to(torch.int64))
            cat["a_excl"].append(d["a_excl"][:ni])
            cat["a_woff"].append(d["a_woff"][:ni] + W)
            cat["t_p0"].append(d["t_p0"][:nt] + P)
            s = d["src"][:rows].to(torch.int64)
            cat["src"].append(torch.where(s < nz[i], s + int(z0[i]),
                                          self.num_zrows + R + (s - nz[i])))
            panel, vpanel = op.panels(precision)
            panels.append(panel[:rows * TILE_ROWS])
            vpanels.append(vpanel[:int(op._vpanel_size)])
            G += ng
            W += int(op._desc.num_work)
            P += rows
            V += int(op._vpanel_size)
            max_gt = max(max_gt, int(op._desc.max_group_tiles))
            needs_zero |= bool(op._needs_zero_z)
        cat["a_woff"].append(torch.tensor([W], dtype=torch.int64, device=dev))
        cat["t_p0"].append(torch.tensor([P], dtype=torch.int64, device=dev))
        i32 = ("g_c0", "g_n", "g_kz", "g_ldv", "a_grp", "a_j0", "a_j1", "src")

        def join(k):
            parts = [p for p in cat[k] if p.numel()]
            dt = torch.int32 if k in i32 else (torch.uint8 if k == "a_excl" else torch.int64)
            if not parts:
                return torch.zeros(1, dtype=dt, device=dev)
            return torch.cat(parts).to(dt).contiguous()
        self._dev = {k: join(k) for k in cat}
        self._panel = torch.cat(panels) if P else torch.zeros(8, dtype=panels[0].dtype,
                                                              device=dev)
        self._vpanel = torch.cat(vpanels) if V else torch.zeros(8, dtype=panels[0].dtype,
                                                                device=dev)
        self._needs_zero_z = needs_zero
        self.panel_rows = P
        desc = fgb_op_desc()
        for k in ("g_c0", "g_n", "g_kz", "g_ldv", "g_voff", "g_z0", "a_grp", "a_j0", "a_j1",
                  "a_excl", "t_p0", "src", "a_woff"):
            setattr(desc, k, self._dev[k].data_ptr())
        desc.num_items = sum(int(op._desc.num_items) for op in ops)
        desc.num_tiles = self.num_rows // TILE_ROWS
        desc.N = self.num_rows
        desc.num_zrows = self.num_zrows
        desc.max_group_tiles = max_gt
        desc.num_work = W
        desc.panel_rows = P
        desc.tile_rows = TILE_ROWS
        self._desc = desc
        # merged cluster row of every facet (meshes concatenated in order)
        cl = []
        for i, op in enumerate(ops):
            inv = torch.empty_like(op._perm_d)
            inv[op._perm_d] = torch.arange(op.num_faces, device=dev, dtype=op._perm_d.dtype)
            cl.append(inv.to(torch.int64) + int(self.row0[i]))
        self.cluster_row = torch.cat(cl)
        self.device = dev

    @property
    def nbytes(self):
        return (self._panel.numel() * self._panel.element_size()
                + self._vpanel.numel() * self._vpanel.element_size())

    def to_cluster(self, x):
        """Facet order (meshes concatenated) -> merged cluster order."""
        shape = (self.num_rows,) + tuple(x.shape[1:])
        out = torch.zeros(shape, dtype=x.dtype, device=x.device)
        out.index_copy_(0, self.cluster_row, x)
        return out

    def from_cluster(self, xp):
        return xp.index_select(0, self.cluster_row)

    def matvec_cluster(self, xp, out=None, z=None, add=None, alpha=1.0):
        """y = F x (or add + alpha F x) in the merged cluster order, K = 1."""
        V = torch.float64 if self.precision == "fp64" else torch.float32
        fn = "fgb_matvec_f64" if self.precision == "fp64" else "fgb_matvec_f32"
        if xp.dtype != V or not xp.is_contiguous():
            xp = xp.to(V).contiguous()
        if out is None:
            out = torch.empty(self.num_rows, dtype=V, device=xp.device)
        if z is None:
            z = torch.empty(max(self.num_zrows, 1), dtype=V, device=xp.device)
        _lib.call(fn, C.byref(self._desc), _lib.ptr(self._panel), _lib.ptr(self._vpanel),
                  _lib.ptr(xp), _lib.ptr(z), _lib.ptr(out), _lib.ptr(add), float(alpha),
                  int(self._needs_zero_z), _lib.stream_handle())
        return out

    def __matmul__(self, x):
        """Facet-order product (meshes concatenated)."""
        return self.from_cluster(self.matvec_cluster(self.to_cluster(x)))


class MultiMeshThermalModel:
    """ThermalModel (model.py:108-234) for many independent meshes at once
    (module docstring), FP32.

    ops: the meshes' CompressedFormFactorMatrix (built on their shape
    models); t (S+1,) uniformly spaced times; D (S+1, 3) sun directions and
    F0 (S+1,) solar constants shared by the meshes; rho, emiss, Fgeotherm
    scalars or per facet (meshes concatenated); z (nz+1,), ti and rhoc
    (nz+1,) shared; T0 scalar or (num_faces, nz+1).  ``run(steps)`` advances
    and returns the surface temperatures of the last step (device, facet
    order); ``T`` gives all profiles."""

    def __init__(self, ops, t, D, F0, rho, z, ti, rhoc, emiss, Fgeotherm, T0,
                 use_graph=True):
        dev = _lib.require_cuda()
        self.op = op = BlockDiagonalOperator(ops, "fp32")
        t = np.asarray(t, np.float64)
        D = np.asarray(D, np.float64)
        if D.ndim != 2 or D.shape[1] != 3 or D.shape[0] != t.size:
            raise ValueError('sun positions ("D") should be an (S+1) x 3 array, one per time')
        dts = np.diff(t)
        if dts.size == 0:
            raise ValueError("need at least two times")
        if use_graph and not np.allclose(dts, dts[0], rtol=1e-12, atol=0):
            raise ValueError("the CUDA-graph path needs uniformly spaced times")
        self.dts = dts
        self.S = dts.size
        F0 = np.broadcast_to(np.asarray(F0, np.float64), (t.size,))
        n, R = op.num_faces, op.num_rows
        z = np.asarray(z, np.float64)
        w = z.size
        f32 = torch.float32

        def facetvec(v, name):
            a = np.asarray(v, np.float64)
            if a.ndim and a.shape != (n,):
                raise ValueError(f'"{name}" should be a scalar or have one value per facet')
            a = np.broadcast_to(a, (n,))
            return op.to_cluster(torch.as_tensor(np.ascontiguousarray(a), dtype=f32,
                                                 device=dev))

        self.rho = facetvec(rho, "rho")
        self.emiss = facetvec(emiss, "emiss")
        # padding rows: a benign facet (unit emissivity, no flux)
        pad = torch.ones(R, dtype=torch.bool, device=dev)
        pad[op.cluster_row] = False
        self.emiss[pad] = 1.0
        self.Fg = facetvec(Fgeotherm, "Fgeotherm")
        self.z = torch.as_tensor(z, dtype=f32, device=dev)
        self.ti = torch.as_tensor(np.broadcast_to(np.asarray(ti, np.float64), (w,)).copy(),
                                  dtype=f32, device=dev)
        self.rhoc = torch.as_tensor(np.broadcast_to(np.asarray(rhoc, np.float64), (w,)).copy(),
                                    dtype=f32, device=dev)
        # insolation of every mesh and step, merged cluster order, one row per step
        E = torch.zeros((t.size, R), dtype=f32, device=dev)
        for i, ffi in enumerate(ops):
            Ei = ffi.shape_model.get_direct_irradiance_batch(F0, D, out_dtype=f32)
            r0 = int(op.row0[i])
            E[:, r0:r0 + ffi.num_faces] = Ei.index_select(0, ffi._perm_d).t()
        self.E = E
        # initial state (model.py:165-171)
        Q0 = (1 - self.rho) * E[0] + self.Fg
        T0a = np.asarray(T0, np.float64)
        if T0a.ndim == 0:
            T = torch.full((R, w), float(T0a), dtype=f32, device=dev)
        else:
            if T0a.shape != (n, w):
                raise ValueError('"T0" should be a scalar or a (num_faces, nz+1) array')
            T = op.to_cluster(torch.as_tensor(T0a, dtype=f32, device=dev))
            T[pad] = 200.0
        self._T = [T.contiguous(), torch.empty_like(T)]
        self._Q = [Q0.contiguous(), torch.empty_like(Q0)]
        self.Tsurf = ((Q0 / (SIGMA * self.emiss))**0.25).contiguous()
        self.Qrefl = torch.zeros(R, dtype=f32, device=dev)
        self.QIR = torch.zeros(R, dtype=f32, device=dev)
        self._Ebuf = [torch.empty(R, dtype=f32, device=dev) for _ in range(2)]
        self._u = torch.empty(R, dtype=f32, device=dev)
        self._y = torch.empty(R, dtype=f32, device=dev)
        self._zs = torch.empty(max(op.num_zrows, 1), dtype=f32, device=dev)
        self._Fsurf = torch.empty(R, dtype=f32, device=dev)
        self.flags = torch.zeros(1, dtype=torch.int32, device=dev)
        self.nz = w - 1
        self.step_index = 0
        self.use_graph = use_graph
        self._graph = None
        self._pad = pad

    # one step: buffers parity p (profiles and fluxes p -> 1 - p), E in _Ebuf[p]
    def _step(self, p, dt):
        op = self.op
        E = self._Ebuf[p]
        torch.add(E, self.Qrefl, out=self._u)
        op.matvec_cluster(self._u, out=self._y, z=self._zs)
        torch.mul(self._y, self.rho, out=self._y)
        torch.clamp(self._y, min=0.0, out=self.Qrefl)           # Qrefl_{n+1}
        # emiss sigma Tsurf^4 + (1 - emiss) QIR
        torch.mul(self.Tsurf, self.Tsurf, out=self._u)
        self._u.mul_(self._u).mul_(self.emiss).mul_(SIGMA)
        self._u.add_(self.QIR * (1 - self.emiss))
        op.matvec_cluster(self._u, out=self._y, z=self._zs)
        torch.clamp(self._y, min=0.0, out=self.QIR)              # QIR_{n+1}
        Qn, Qnp1 = self._Q[p], self._Q[1 - p]
        torch.add(E, self.Qrefl, out=Qnp1)
        Qnp1.mul_(1 - self.rho).add_(self.emiss * self.QIR)
        Tin, Tout = self._T[p], self._T[1 - p]
        _lib.call("fgb_conduction_q_f32", op.num_rows, self.nz, _lib.ptr(self.z), float(dt),
                  _lib.ptr(Qn), _lib.ptr(Qnp1), _lib.ptr(Tin), _lib.ptr(Tout), _lib.ptr(self.ti),
                  _lib.ptr(self.rhoc), _lib.ptr(self.emiss), _lib.ptr(self.Fg),
                  _lib.ptr(self._Fsurf), _lib.ptr(self.flags), _lib.stream_handle())
        self.Tsurf.copy_(Tout[:, 0])

    def _capture(self):
        """Record two steps (parities 0 then 1) in one CUDA graph.  Capture
        records the launches without running them; the first two steps of
        ``run`` are eager, so every kernel has been loaded and launched once
        before."""
        g = torch.cuda.CUDAGraph()
        dt = float(self.dts[0])
        with torch.cuda.graph(g):
            self._step(0, dt)
            self._step(1, dt)
        return g

    def run(self, steps=None):
        """Advance ``steps`` steps (default: all that remain); returns the
        surface temperatures (device, facet order)."""
        left = self.S - self.step_index
        steps = left if steps is None else min(int(steps), left)
        i = self.step_index
        end = i + steps
        while i < end:
            if self.use_graph and i >= 2 and i % 2 == 0 and end - i >= 2:
                if self._graph is None:
                    self._graph = self._capture()
                self._Ebuf[0].copy_(self.E[i + 1])
                self._Ebuf[1].copy_(self.E[i + 2])
                self._graph.replay()
                i += 2
            else:
                p = i % 2
                self._Ebuf[p].copy_(self.E[i + 1])
                self._step(p, float(self.dts[i]))
                i += 1
            self.step_index = i
        return self.surface_temperature()

    def check_errors(self):
        f = int(self.flags.item())
        if f & _lib.FLAG_ZERO_PIVOT:
            raise RuntimeError("tridag failed")
        if f & (_lib.FLAG_NONFINITE_IN | _lib.FLAG_NONFINITE_OUT):
            raise RuntimeError("computed nonfinite temperatures while stepping")
        if f & (_lib.FLAG_NEGATIVE_IN | _lib.FLAG_NEGATIVE_OUT):
            raise RuntimeError("computed negative temperatures while stepping")

    @property
    def T(self):
        """Profiles (num_faces, nz+1) in facet order (meshes concatenated)."""
        return self.op.from_cluster(self._T[self.step_index % 2])

    def surface_temperature(self):
        return self.op.from_cluster(self._T[self.step_index % 2][:, 0].contiguous())
