"""CPU: the offset arithmetic of BlockDiagonalOperator (fluxpy_gb300/batch.py)
on synthetic panel layouts.  A plain restatement of the two-phase panel
product (the layout documented in fluxpy_gb300/csrc/matvec.cu) applied to the
merged layout must equal each operator's own product, mesh by mesh; the
GPU test (test_gpu_batch.py) checks the kernels on real operators."""
from types import SimpleNamespace

import numpy as np
import torch

from fluxpy_gb300.batch import BlockDiagonalOperator

TILE = 64


class FakeOp:
    """A random but valid panel layout for an operator on N facets."""

    def __init__(self, rng, N):
        self.num_faces = N
        self._perm_d = torch.as_tensor(rng.permutation(N))
        ng = int(rng.integers(0, 6))
        g_c0, g_n, g_kz = [], [], []
        for _ in range(ng):
            n = int(rng.integers(1, min(N, 150) + 1))
            g_c0.append(int(rng.integers(0, N - n + 1)))
            g_n.append(n)
            g_kz.append(int(rng.integers(1, 9)))
        g_ldv = [(n + 7) // 8 * 8 for n in g_n]
        g_voff = np.concatenate([[0], np.cumsum(np.multiply(g_kz, g_ldv))]).astype(np.int64)
        g_z0 = np.concatenate([[0], np.cumsum(g_kz)]).astype(np.int64)
        self._num_zrows = int(g_z0[-1])
        # items: whole groups, or a group split in two column ranges
        a_grp, a_j0, a_j1, a_ex = [], [], [], []
        for g in range(ng):
            if g_n[g] > 2 and rng.random() < 0.5:
                cut = int(rng.integers(1, g_n[g]))
                for j0, j1 in ((0, cut), (cut, g_n[g])):
                    a_grp.append(g); a_j0.append(j0); a_j1.append(j1); a_ex.append(0)
            else:
                a_grp.append(g); a_j0.append(0); a_j1.append(g_n[g]); a_ex.append(1)
        a_woff = np.concatenate([[0], np.cumsum([(g_kz[g] + 63) // 64 for g in a_grp])])
        vpanel = np.zeros(int(g_voff[-1]))
        for g in range(ng):
            blk = rng.uniform(-1, 1, (g_kz[g], g_ldv[g]))
            blk[:, g_n[g]:] = 0
            vpanel[g_voff[g]:g_voff[g + 1]] = blk.ravel()
        ntiles = (N + TILE - 1) // TILE
        L = rng.integers(0, 3, ntiles) * TILE
        t_p0 = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
        P = int(t_p0[-1])
        src = rng.integers(0, self._num_zrows + N, P)
        panel = rng.uniform(-1, 1, (P, TILE))
        for t in range(ntiles):
            valid = min(TILE, N - t * TILE)
            panel[t_p0[t]:t_p0[t + 1], valid:] = 0
        self._panel_rows = P
        self._vpanel_size = int(g_voff[-1])
        self._needs_zero_z = not all(a_ex)

        def d(a, dt):
            a = np.asarray(a, dtype=dt)
            return torch.as_tensor(a if a.size else np.zeros(1, dt))
        self._dev = dict(g_c0=d(g_c0, np.int32), g_n=d(g_n, np.int32), g_kz=d(g_kz, np.int32),
                         g_ldv=d(g_ldv, np.int32), g_voff=d(g_voff[:-1], np.int64),
                         g_z0=d(g_z0[:-1], np.int64), a_grp=d(a_grp, np.int32),
                         a_j0=d(a_j0, np.int32), a_j1=d(a_j1, np.int32), a_excl=d(a_ex, np.uint8),
                         a_woff=d(a_woff, np.int64), t_p0=d(t_p0, np.int64),
                         src=d(src, np.int32))
        self._desc = SimpleNamespace(num_items=len(a_grp), num_tiles=ntiles,
                                     num_work=int(a_woff[-1]), max_group_tiles=1)
        self.stats = {"groups": ng}
        self._pn = (torch.as_tensor(panel.ravel() if P else np.zeros(8)),
                    torch.as_tensor(vpanel if vpanel.size else np.zeros(8)))

    def panels(self, precision):
        return self._pn


def panel_product(dev, num_items, ntiles, panel, vpanel, nrows, num_zrows, x):
    """y = F x for the panel layout (phase A, then phase B)."""
    z = np.zeros(num_zrows)
    for i in range(num_items):
        g = int(dev["a_grp"][i])
        j0, j1 = int(dev["a_j0"][i]), int(dev["a_j1"][i])
        kz, ldv = int(dev["g_kz"][g]), int(dev["g_ldv"][g])
        c0, voff, z0 = int(dev["g_c0"][g]), int(dev["g_voff"][g]), int(dev["g_z0"][g])
        V = vpanel[voff:voff + kz * ldv].reshape(kz, ldv)
        z[z0:z0 + kz] += V[:, j0:j1] @ x[c0 + j0:c0 + j1]
    S = np.concatenate([z, x])
    y = np.zeros(nrows)
    W = panel.reshape(-1, TILE) if panel.size >= TILE else np.zeros((0, TILE))
    for t in range(ntiles):
        p0, p1 = int(dev["t_p0"][t]), int(dev["t_p0"][t + 1])
        rows = min(TILE, nrows - t * TILE)
        for l in range(p0, p1):
            y[t * TILE:t * TILE + rows] += W[l, :rows] * S[int(dev["src"][l])]
    return y


def test_merged_layout_product_equals_each_operator():
    rng = np.random.default_rng(11)
    ops = [FakeOp(rng, N) for N in (70, 200, 1, 130, 64, 300)]
    bd = BlockDiagonalOperator(ops, "fp64")
    assert bd.num_rows == sum((op.num_faces + 63) // 64 * 64 for op in ops)
    assert bd.num_zrows == sum(op._num_zrows for op in ops)
    x = rng.uniform(-1, 1, bd.num_faces)
    dv = {k: v.numpy() for k, v in bd._dev.items()}
    xc = bd.to_cluster(torch.as_tensor(x)).numpy()
    yc = panel_product(dv, bd._desc.num_items, bd._desc.num_tiles, bd._panel.numpy(),
                       bd._vpanel.numpy(), bd.num_rows, bd.num_zrows, xc)
    y = bd.from_cluster(torch.as_tensor(yc)).numpy()
    o = 0
    for op in ops:
        perm = op._perm_d.numpy()
        xi = x[o:o + op.num_faces]
        d_op = {k: v.numpy() for k, v in op._dev.items()}
        yp = panel_product(d_op, op._desc.num_items, op._desc.num_tiles, op._pn[0].numpy(),
                           op._pn[1].numpy(), op.num_faces, op._num_zrows, xi[perm])
        yi = np.empty(op.num_faces)
        yi[perm] = yp
        assert np.allclose(y[o:o + op.num_faces], yi, rtol=1e-13, atol=1e-13)
        o += op.num_faces
    # rows past a mesh's facets are padding and stay zero
    pad = np.ones(bd.num_rows, bool)
    pad[bd.cluster_row.numpy()] = False
    assert not yc[pad].any()
    assert bd._needs_zero_z == any(op._needs_zero_z for op in ops)
