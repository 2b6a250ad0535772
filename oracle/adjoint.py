"""ORACLE — FP64 CPU restatement of the conduction step with per-facet
thermal inertia, its reverse-mode derivative, and the coupled
radiosity + conduction misfit with its gradient (test infrastructure only;
the product never imports this module).

* ``pcc_q_forward`` restates src/flux/pcc/conductionQ.c:10-186 (with the
  Thomas solve of src/flux/pcc/tridag.c:5-34) vectorised over facets, with
  ``ti`` given per facet and layer (num_faces, nz+1).  Every operation keeps
  the reference's order, so with equal rows of ``ti`` the result is
  bit-identical to the reference's per-facet C routine.
* ``pcc_q_adjoint`` is the transpose of that step's Jacobian, taken through
  every predictor-corrector pass (conductionQ.c:103-172: the linearisation
  temperature of a redo depends on the previous pass's surface value) and
  applied to a cotangent of the output profile.
* ``coupled_forward`` / ``coupled_gradient``: the misfit model differentiated
  by the GPU adjoint, with a dense form-factor matrix.  Per step n >= 1:
      B_n    = solve (I - F diag(rho)) B = E_n       (solve.py:36-45, 'right')
      QIR_n  = F (emiss sigma Ts_{n-1}^4 + (1 - emiss) QIR_{n-1})   (model.py:44-69)
      Q_n    = (1 - rho) B_n + emiss QIR_n
      T_n    = conductionQ(T_{n-1}, Q_{n-1}, Q_n; emiss, ti)
      L     += 0.5 sum_i (T_n[i, 0] - Tobs_n[i])^2
  with Q_0 = (1 - rho) B_0 + Fgeotherm, Ts_0 = (Q_0 / (sigma emiss))^(1/4)
  and QIR_0 = 0, the initial state of model.py:165-171.  The gradient is a
  plain reverse sweep over stored states (no checkpointing: this is the
  checker, sized for a few thousand facets).
"""
from __future__ import annotations

import numpy as np
from scipy.constants import Stefan_Boltzmann as SIGMA_MODEL

SIGMA_PCC = 5.6704e-8   # conductionQ.c:55


# ---------------------------------------------------------------- grid ----
def _grid(z, dt, ti, rhoc):
    """Per-facet alpha, gamma (N, nz+1) and k1/dz (N,), conductionQ.c:69-83
    in the reference's order of operations; also the layer constants of
    their derivatives with respect to k."""
    nz = z.size - 1
    N = ti.shape[0]
    k = ti * ti / rhoc[None, :]
    dz = 2. * z[1]
    beta = dt / rhoc[1] / (2. * dz * dz)
    alpha = np.zeros((N, nz + 1))
    gamma = np.zeros((N, nz + 1))
    ca = np.zeros(nz + 1)   # d alpha_i / d k_{i+1}
    cg = np.zeros(nz + 1)   # d gamma_i / d k_i
    alpha[:, 1] = beta * k[:, 2]
    gamma[:, 1] = beta * k[:, 1]
    ca[1] = beta
    cg[1] = beta
    for i in range(2, nz):
        buf = dt / (z[i + 1] - z[i - 1])
        alpha[:, i] = 2 * k[:, i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i])
        gamma[:, i] = 2 * k[:, i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1])
        ca[i] = 2 * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i])
        cg[i] = 2 * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1])
    buf = dt / (z[nz] - z[nz - 1]) / (z[nz] - z[nz - 1])
    gamma[:, nz] = k[:, nz] * buf / (2 * rhoc[nz])
    cg[nz] = buf / (2 * rhoc[nz])
    kappa = k[:, 1] / dz
    return k, alpha, gamma, kappa, ca, cg, dz


def _pass(nz, Tpre, Tr, Qn, Qnp1, em, alpha, gamma, kappa, rhs_bottom):
    """One linearised pass (conductionQ.c:103-157): returns u (N, nz+1),
    the Thomas factors, T0 and the boundary quantities."""
    N = Tpre.shape[0]
    arad = -3 * em * SIGMA_PCC * Tr * Tr * Tr * Tr
    brad = 2 * em * SIGMA_PCC * Tr * Tr * Tr
    ann = (Qn - arad) / (kappa + brad)
    annp1 = (Qnp1 - arad) / (kappa + brad)
    bn = (kappa - brad) / (kappa + brad)
    a1, g1 = alpha[:, 1], gamma[:, 1]
    b1 = 1. + a1 + g1 - g1 * bn
    r = np.zeros((N, nz + 1))
    r[:, 1] = g1 * (annp1 + ann) + (1. - a1 - g1 + g1 * bn) * Tpre[:, 1] + a1 * Tpre[:, 2]
    for i in range(2, nz):
        r[:, i] = (gamma[:, i] * Tpre[:, i - 1] + (1 - alpha[:, i] - gamma[:, i]) * Tpre[:, i]
                   + alpha[:, i] * Tpre[:, i + 1])
    r[:, nz] = gamma[:, nz] * Tpre[:, nz - 1] + (1. - gamma[:, nz]) * Tpre[:, nz] + rhs_bottom
    # tridag.c:18-30 with a_i = -gamma_i, b_i = 1 + alpha_i + gamma_i
    # (b_nz = 1 + gamma_nz, b_1 above), c_i = -alpha_i
    u = np.zeros((N, nz + 1))
    gam = np.zeros((N, nz + 1))
    bet = b1.copy()
    u[:, 1] = r[:, 1] / bet
    for j in range(2, nz + 1):
        gam[:, j] = (-alpha[:, j - 1]) / bet
        bj = (1. + gamma[:, nz]) if j == nz else (1. + alpha[:, j] + gamma[:, j])
        bet = bj - (-gamma[:, j]) * gam[:, j]
        u[:, j] = (r[:, j] - (-gamma[:, j]) * u[:, j - 1]) / bet
    for j in range(nz - 1, 0, -1):
        u[:, j] -= gam[:, j + 1] * u[:, j + 1]
    T0 = 0.5 * (annp1 + bn * u[:, 1] + u[:, 1])
    return dict(u=u, T0=T0, arad=arad, brad=brad, ann=ann, annp1=annp1, bn=bn, b1=b1)


def pcc_q_forward(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Fgeotherm, record=False):
    """One conductionQ step for every facet (FP64).  ``T`` (N, nz+1) is not
    modified; returns the new profiles, and with ``record`` also the
    linearisation temperatures of every pass (list) and the pass count."""
    z = np.asarray(z, np.float64)
    rhoc = np.asarray(rhoc, np.float64)
    T = np.asarray(T, np.float64)
    N, w = T.shape
    nz = w - 1
    ti = np.broadcast_to(np.asarray(ti, np.float64), (N, w))
    k, alpha, gamma, kappa, _, _, _ = _grid(z, dt, ti, rhoc)
    rhs_bottom = dt / rhoc[nz] * Fgeotherm / (z[nz] - z[nz - 1])
    Tr = T[:, 0].copy()
    out = np.empty_like(T)
    done = np.zeros(N, bool)
    npass = np.zeros(N, np.int64)
    trs = []
    it = 0
    while True:
        trs.append(Tr.copy())
        p = _pass(nz, T, Tr, Qn, Qnp1, emiss, alpha, gamma, kappa, rhs_bottom)
        T0 = p["T0"]
        redo = ((T0 > 1.2 * Tr) | (T0 < 0.8 * Tr)) & (it < 10) & ~done
        fin = ~done & ~redo
        out[fin, 0] = T0[fin]
        out[fin, 1:] = p["u"][fin, 1:]
        npass[fin] = it
        done |= fin
        if done.all():
            break
        it += 1
        Tr = np.where(redo, np.sqrt(Tr * T0), Tr)
    if record:
        return out, trs, npass
    return out


def pcc_q_adjoint(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Fgeotherm, gT):
    """Reverse-mode derivative of ``pcc_q_forward``: given the cotangent gT
    of the new profiles, returns (gT_pre, gQn, gQnp1, gemiss, gti) with
    gti of shape (N, nz+1) (gti[:, 0] = 0: ti[0] is not used)."""
    z = np.asarray(z, np.float64)
    rhoc = np.asarray(rhoc, np.float64)
    T = np.asarray(T, np.float64)
    N, w = T.shape
    nz = w - 1
    ti = np.broadcast_to(np.asarray(ti, np.float64), (N, w))
    _, trs, npass = pcc_q_forward(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Fgeotherm, record=True)
    k, alpha, gamma, kappa, ca, cg, dz = _grid(z, dt, ti, rhoc)
    rhs_bottom = dt / rhoc[nz] * Fgeotherm / (z[nz] - z[nz - 1])
    em = np.asarray(emiss, np.float64)
    gTpre = np.zeros((N, w))
    galpha = np.zeros((N, w))
    ggamma = np.zeros((N, w))
    gkappa = np.zeros(N)
    gQn = np.zeros(N)
    gQnp1 = np.zeros(N)
    gem = np.zeros(N)
    gT0 = np.zeros(N)
    gu = np.zeros((N, w))
    gTr_next = np.zeros(N)
    T0_prev = None
    for p in range(int(npass.max()), -1, -1):
        act = npass >= p
        final = npass == p
        Tr = trs[p]
        fw = _pass(nz, T, Tr, Qn, Qnp1, em, alpha, gamma, kappa, rhs_bottom)
        u, bn, b1 = fw["u"], fw["bn"], fw["b1"]
        # seeds of this pass: the step's output on its final pass; on an
        # earlier pass, T0 only (through the next pass's Tr)
        gT0 = np.where(final, gT[:, 0], 0.0)
        gu = np.where(final[:, None], gT, 0.0)
        gu[:, 0] = 0.0
        if p < int(npass.max()):
            # Tr_{p+1} = sqrt(Tr_p T0_p)
            nxt = ~final & act
            Tr1 = trs[p + 1]
            gT0 = gT0 + np.where(nxt, gTr_next * Tr1 / (2 * fw["T0"]), 0.0)
            gTr_carry = np.where(nxt, gTr_next * Tr1 / (2 * Tr), 0.0)
        else:
            gTr_carry = np.zeros(N)
        gT0 = np.where(act, gT0, 0.0)
        # T0 = 0.5 (annp1 + bn u1 + u1)
        g_annp1 = 0.5 * gT0
        g_bn = 0.5 * u[:, 1] * gT0
        gu[:, 1] += 0.5 * (bn + 1) * gT0
        # g_r = M^-T gu; M^T: diag b, sub (i, i-1) = c_{i-1} = -alpha_{i-1},
        # super (i, i+1) = a_{i+1} = -gamma_{i+1}
        bdiag = np.empty((N, w))
        bdiag[:, 1] = b1
        for i in range(2, nz):
            bdiag[:, i] = 1. + alpha[:, i] + gamma[:, i]
        bdiag[:, nz] = 1. + gamma[:, nz]
        gr = _tridiag_T(nz, alpha, gamma, bdiag, gu)
        # M entries: g_b_i = -gr_i u_i, g_a_i = -gr_i u_{i-1}, g_c_i = -gr_i u_{i+1}
        gb = -gr * u
        g_a = np.zeros((N, w))
        g_c = np.zeros((N, w))
        g_a[:, 2:] = -gr[:, 2:] * u[:, 1:nz]
        g_c[:, 1:nz] = -gr[:, 1:nz] * u[:, 2:]
        ga = np.zeros((N, w))
        gg = np.zeros((N, w))
        # row 1: b1 = 1 + a1 + g1 - g1 bn, c1 = -a1
        ga[:, 1] += gb[:, 1] - g_c[:, 1]
        gg[:, 1] += gb[:, 1] * (1 - bn)
        g_bn += -gamma[:, 1] * gb[:, 1]
        for i in range(2, nz):
            ga[:, i] += gb[:, i] - g_c[:, i]
            gg[:, i] += gb[:, i] - g_a[:, i]
        gg[:, nz] += gb[:, nz] - g_a[:, nz]
        # right-hand side r (pre-step profile Tpre)
        Tp = T
        g1 = gamma[:, 1]
        a1 = alpha[:, 1]
        ann, annp1 = fw["ann"], fw["annp1"]
        gg[:, 1] += gr[:, 1] * ((annp1 + ann) + (bn - 1) * Tp[:, 1])
        ga[:, 1] += gr[:, 1] * (Tp[:, 2] - Tp[:, 1])
        g_bn += gr[:, 1] * g1 * Tp[:, 1]
        g_annp1 += gr[:, 1] * g1
        g_ann = gr[:, 1] * g1
        gTp = np.zeros((N, w))
        gTp[:, 1] += gr[:, 1] * (1. - a1 - g1 + g1 * bn)
        gTp[:, 2] += gr[:, 1] * a1
        for i in range(2, nz):
            gg[:, i] += gr[:, i] * (Tp[:, i - 1] - Tp[:, i])
            ga[:, i] += gr[:, i] * (Tp[:, i + 1] - Tp[:, i])
            gTp[:, i - 1] += gr[:, i] * gamma[:, i]
            gTp[:, i] += gr[:, i] * (1 - alpha[:, i] - gamma[:, i])
            gTp[:, i + 1] += gr[:, i] * alpha[:, i]
        gg[:, nz] += gr[:, nz] * (Tp[:, nz - 1] - Tp[:, nz])
        gTp[:, nz - 1] += gr[:, nz] * gamma[:, nz]
        gTp[:, nz] += gr[:, nz] * (1 - gamma[:, nz])
        # boundary quantities -> Tr, emiss, kappa, Qn, Qnp1
        D = kappa + fw["brad"]
        gQn_p = g_ann / D
        gQnp1_p = g_annp1 / D
        g_arad = -(g_ann + g_annp1) / D
        g_D = -(g_ann * ann + g_annp1 * annp1 + g_bn * bn) / D
        gkap = g_bn / D + g_D
        g_brad = -g_bn / D + g_D
        gem_p = g_arad * (-3 * SIGMA_PCC * Tr**4) + g_brad * (2 * SIGMA_PCC * Tr**3)
        gTr = (g_arad * (-12 * em * SIGMA_PCC * Tr**3) + g_brad * (6 * em * SIGMA_PCC * Tr**2)
               + gTr_carry)
        m = act.astype(np.float64)
        gTpre += gTp * m[:, None]
        galpha += ga * m[:, None]
        ggamma += gg * m[:, None]
        gkappa += gkap * m
        gQn += gQn_p * m
        gQnp1 += gQnp1_p * m
        gem += gem_p * m
        gTr_next = gTr * m
    gTpre[:, 0] += gTr_next
    # alpha, gamma, kappa -> k -> ti
    gk = np.zeros((N, w))
    for i in range(1, nz):
        gk[:, i + 1] += galpha[:, i] * ca[i]
    for i in range(1, nz + 1):
        gk[:, i] += ggamma[:, i] * cg[i]
    gk[:, 1] += gkappa / dz
    gti = np.zeros((N, w))
    gti[:, 1:] = gk[:, 1:] * 2 * ti[:, 1:] / rhoc[None, 1:]
    return gTpre, gQn, gQnp1, gem, gti


def _tridiag_T(nz, alpha, gamma, bdiag, rhs):
    """Solve M^T x = rhs (rows 1..nz) for the conduction matrix M."""
    N = rhs.shape[0]
    x = np.zeros((N, nz + 1))
    gam = np.zeros((N, nz + 1))
    bet = bdiag[:, 1].copy()
    x[:, 1] = rhs[:, 1] / bet
    for j in range(2, nz + 1):
        sub = -alpha[:, j - 1]        # M^T[j, j-1] = M[j-1, j] = c_{j-1}
        sup_prev = -gamma[:, j]       # M^T[j-1, j] = M[j, j-1] = a_j
        gam[:, j] = sup_prev / bet
        bet = bdiag[:, j] - sub * gam[:, j]
        x[:, j] = (rhs[:, j] - sub * x[:, j - 1]) / bet
    for j in range(nz - 1, 0, -1):
        x[:, j] -= gam[:, j + 1] * x[:, j + 1]
    return x


# ------------------------------------------------------ coupled model ----
def _solve_right(F, E, rho, tol=1e-14, max_iter=10000):
    """B = E + F (rho B) for every column of E, to a relative update of tol."""
    B = E.copy()
    for _ in range(max_iter):
        B1 = E + F @ (rho[:, None] * B if B.ndim == 2 else rho * B)
        if np.abs(B1 - B).max() <= tol * max(np.abs(E).max(), 1e-300):
            return B1
        B = B1
    raise RuntimeError("no convergence")


def _solve_right_T(F, G, rho, tol=1e-14, max_iter=10000):
    """lam = G + rho (F^T lam) for every column of G."""
    L = G.copy()
    FT = F.T
    for _ in range(max_iter):
        L1 = G + rho[:, None] * (FT @ L)
        if np.abs(L1 - L).max() <= tol * max(np.abs(G).max(), 1e-300):
            return L1
        L = L1
    raise RuntimeError("no convergence")


def coupled_forward(F, E, rho, emiss, ti, z, rhoc, dt, T0, Fgeotherm, Tobs, store=False):
    """Misfit of the coupled model (module docstring).  E (N, S+1): the
    direct insolation at steps 0..S; Tobs (N, S); ti per facet (N,) uniform
    with depth, or (N, nz+1)."""
    N, S1 = E.shape
    S = S1 - 1
    w = z.size
    tif = np.broadcast_to(ti[:, None] if np.ndim(ti) == 1 else ti, (N, w))
    B = _solve_right(F, E, rho)
    Q = (1 - rho) * B[:, 0] + Fgeotherm
    Ts = (Q / (SIGMA_MODEL * emiss))**0.25
    QIR = np.zeros(N)
    T = np.array(T0, np.float64, copy=True)
    L = 0.0
    states = []
    for n in range(1, S + 1):
        QIRn = F @ (emiss * SIGMA_MODEL * Ts**4 + (1 - emiss) * QIR)
        Qn1 = (1 - rho) * B[:, n] + emiss * QIRn
        if store:
            states.append((T.copy(), Q.copy(), Qn1.copy(), Ts.copy(), QIR.copy(), QIRn.copy()))
        T = pcc_q_forward(z, dt, Q, Qn1, T, tif, rhoc, emiss, Fgeotherm)
        Ts = T[:, 0].copy()
        L += 0.5 * np.sum((Ts - Tobs[:, n - 1])**2)
        Q, QIR = Qn1, QIRn
    if store:
        return L, B, states, T
    return L


def coupled_gradient(F, E, rho, emiss, ti, z, rhoc, dt, T0, Fgeotherm, Tobs):
    """(L, dL/drho, dL/demiss, dL/dti) of ``coupled_forward`` (ti per facet)."""
    N, S1 = E.shape
    S = S1 - 1
    w = z.size
    per_facet = np.ndim(ti) == 1
    tif = np.broadcast_to(ti[:, None] if per_facet else ti, (N, w))
    L, B, states, _ = coupled_forward(F, E, rho, emiss, ti, z, rhoc, dt, T0, Fgeotherm, Tobs,
                                      store=True)
    grho = np.zeros(N)
    gem = np.zeros(N)
    gti = np.zeros((N, w))
    gB = np.zeros((N, S1))
    gT = np.zeros((N, w))
    gQ_next = np.zeros(N)     # cotangent of Q_n through step n+1's Qn argument
    gQIR_next = np.zeros(N)   # cotangent of QIR_n through QIR_{n+1}
    for n in range(S, 0, -1):
        Tprev, Qprev, Qn1, Tsprev, QIRprev, QIRn = states[n - 1]
        Tn_surf = (pcc_q_forward(z, dt, Qprev, Qn1, Tprev, tif, rhoc, emiss, Fgeotherm)[:, 0])
        gT[:, 0] += Tn_surf - Tobs[:, n - 1]
        gTp, gQa, gQb, gem_c, gti_c = pcc_q_adjoint(z, dt, Qprev, Qn1, Tprev, tif, rhoc, emiss,
                                                    Fgeotherm, gT)
        gem += gem_c
        gti += gti_c
        gQn = gQb + gQ_next
        gQ_next = gQa
        gB[:, n] += (1 - rho) * gQn
        grho -= B[:, n] * gQn
        gem += QIRn * gQn
        gQIR = emiss * gQn + gQIR_next
        gu = F.T @ gQIR
        gem += (SIGMA_MODEL * Tsprev**4 - QIRprev) * gu
        gTs = 4 * emiss * SIGMA_MODEL * Tsprev**3 * gu
        gQIR_next = (1 - emiss) * gu
        gT = gTp
        if n > 1:
            gT[:, 0] += gTs
        else:
            # Ts_0 = (Q_0 / (sigma emiss))^(1/4)
            gQ_next = gQ_next + gTs * 0.25 * Tsprev / Qprev
            gem += gTs * (-0.25) * Tsprev / emiss
    # Q_0 = (1 - rho) B_0 + Fgeotherm
    gB[:, 0] += (1 - rho) * gQ_next
    grho -= B[:, 0] * gQ_next
    lam = _solve_right_T(F, gB, rho)
    grho += np.sum(B * (F.T @ lam), axis=1)
    if per_facet:
        return L, grho, gem, gti.sum(axis=1)
    return L, grho, gem, gti
