"""The oracle's conduction adjoint and coupled-model gradient (CPU).

Pins oracle/adjoint.py before the GPU adjoint is compared with it:
* its per-facet-ti conduction step equals the C restatement of
  conductionQ (src/flux/pcc/conductionQ.c:10-186) bit for bit when every
  facet has the same ti, including facets that take predictor-corrector
  redos;
* its reverse-mode step matches central finite differences for every input;
* the coupled radiosity + conduction misfit gradient matches central
  finite differences on random facets.
"""
import numpy as np
import pytest

from oracle import adjoint as A
from oracle import pcc as opcc
from oracle import vis
from fluxpy_gb300 import terrain
from fluxpy_gb300.thermal import setgrid


def _case(N=48, seed=0):
    rng = np.random.default_rng(seed)
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    w = z.size
    T = rng.uniform(150, 300, (N, w))
    ti = np.linspace(55, 400, w)
    rhoc = np.full(w, 1.2e6)
    em = rng.uniform(0.9, 0.98, N)
    Fg = np.full(N, 0.02)
    Qn = rng.uniform(0, 800, N)
    Qnp1 = rng.uniform(0, 800, N)
    # strong cooling or heating: predictor-corrector redos
    Qn[:6], Qnp1[:6] = 1200.0, 0.0
    Qn[6:10], Qnp1[6:10] = 0.0, 3000.0
    T[6:10] = 40.0
    return rng, z, T, ti, rhoc, em, Fg, Qn, Qnp1


def test_forward_equals_c_restatement_bitwise():
    rng, z, T, ti, rhoc, em, Fg, Qn, Qnp1 = _case()
    out, _, npass = A.pcc_q_forward(z, 3600.0, Qn, Qnp1, T, ti, rhoc, em, Fg, record=True)
    ref = T.copy()
    opcc.step_q(z, 3600.0, Qn, Qnp1, ref, ti, rhoc, em, Fg)
    assert np.array_equal(out, ref)
    assert npass.max() >= 1, "the case should exercise predictor-corrector redos"


@pytest.mark.parametrize("which", ["T", "Qn", "Qnp1", "emiss", "ti"])
def test_step_adjoint_matches_finite_differences(which):
    rng, z, T, ti, rhoc, em, Fg, Qn, Qnp1 = _case()
    N, w = T.shape
    tif = np.tile(ti, (N, 1)) * rng.uniform(0.7, 1.3, (N, 1))
    gT = rng.standard_normal((N, w))
    dt = 3600.0
    args = dict(T=T, Qn=Qn, Qnp1=Qnp1, emiss=em, ti=tif)

    def loss(a):
        out = A.pcc_q_forward(z, dt, a["Qn"], a["Qnp1"], a["T"], a["ti"], rhoc, a["emiss"], Fg)
        return np.sum(gT * out, axis=1)   # per facet: facets are independent

    g = dict(zip(["T", "Qn", "Qnp1", "emiss", "ti"],
                 A.pcc_q_adjoint(z, dt, Qn, Qnp1, T, tif, rhoc, em, Fg, gT)))
    x = args[which]
    cols = [0, 1, 2, 7, 20, w - 2, w - 1] if x.ndim == 2 else [None]
    for c in cols:
        if which == "ti" and c == 0:
            continue
        sl = (slice(None), c) if c is not None else slice(None)
        h = 1e-6 * np.abs(x[sl]).max()
        xp, xm = x.copy(), x.copy()
        xp[sl] += h
        xm[sl] -= h
        fd = (loss({**args, which: xp}) - loss({**args, which: xm})) / (2 * h)
        err = np.abs(fd - g[which][sl]).max() / np.abs(fd).max()
        assert err < 1e-6, (which, c, err)


def test_coupled_gradient_matches_finite_differences():
    V, F = terrain.fbm_terrain(n=10, seed=4, n_craters=1)
    P, Nn, Ar = vis.geometry(V, F)
    FF = vis.Scene(V, F).ff_csr(P, Nn, Ar).toarray()
    N = FF.shape[0]
    rng = np.random.default_rng(4)
    S = 8
    dirs = terrain.random_sun_directions(S + 1, seed=2, elev=(5, 40))
    E = np.stack([1365 * np.maximum(0, Nn @ d) for d in dirs], 1)
    z = np.concatenate([[0.0], setgrid(20, 1.1, 0.5)])
    w = z.size
    rhoc = np.full(w, 1.2e6)
    rho = rng.uniform(0.07, 0.2, N)
    em = rng.uniform(0.9, 0.98, N)
    ti = rng.uniform(40, 120, N)
    T0 = np.full((N, w), 200.0)
    Fg = np.full(N, 0.02)
    Tobs = rng.uniform(150, 300, (N, S))
    L, grho, gem, gti = A.coupled_gradient(FF, E, rho, em, ti, z, rhoc, 3600.0, T0, Fg, Tobs)
    grads = dict(rho=grho, emiss=gem, ti=gti)
    base = dict(rho=rho, emiss=em, ti=ti)
    for key, x in base.items():
        for i in rng.choice(N, 4, replace=False):
            h = 1e-5 * x[i]
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            Lp = A.coupled_forward(FF, E, **{**base, key: xp}, z=z, rhoc=rhoc, dt=3600.0,
                                   T0=T0, Fgeotherm=Fg, Tobs=Tobs)
            Lm = A.coupled_forward(FF, E, **{**base, key: xm}, z=z, rhoc=rhoc, dt=3600.0,
                                   T0=T0, Fgeotherm=Fg, Tobs=Tobs)
            fd = (Lp - Lm) / (2 * h)
            assert abs(fd - grads[key][i]) <= 1e-6 * abs(fd), (key, i, fd, grads[key][i])


@pytest.mark.parametrize("nz", [2, 40])
def test_many_redos_and_the_smallest_grid(nz):
    """Up to 8 predictor-corrector redos per step (tiny surface temperature
    with a large flux, a day-long step) and nz = 2: forward bit-identical to
    the C restatement, adjoint equal to central differences."""
    z = np.concatenate([[0.0], setgrid(nz, 1.0817 if nz > 2 else 1.0, 1.0 if nz > 2 else 0.1)])
    w = z.size
    N = 6
    T = np.full((N, w), 200.0)
    T[:, 0] = [1.0, 5.0, 20.0, 200.0, 400.0, 50.0]
    ti, rhoc = np.full(w, 100.0), np.full(w, 1.2e6)
    em, Fg = np.full(N, 0.95), np.full(N, 0.02)
    Qn = np.array([5000.0, 3000.0, 2000.0, 0.0, 0.0, 1000.0])
    Qnp1 = 1.1 * Qn
    dt = 86400.0
    out, _, npass = A.pcc_q_forward(z, dt, Qn, Qnp1, T, ti, rhoc, em, Fg, record=True)
    ref = T.copy()
    opcc.step_q(z, dt, Qn, Qnp1, ref, ti, rhoc, em, Fg)
    assert np.array_equal(out, ref)
    assert npass.max() >= 6
    gT = np.random.default_rng(0).standard_normal((N, w))
    g = A.pcc_q_adjoint(z, dt, Qn, Qnp1, T, np.tile(ti, (N, 1)), rhoc, em, Fg, gT)

    def loss(q):
        return np.sum(gT * A.pcc_q_forward(z, dt, q, Qnp1, T, ti, rhoc, em, Fg), axis=1)
    fd = (loss(Qn + 1e-4) - loss(Qn - 1e-4)) / 2e-4
    assert np.all(np.abs(fd - g[1]) <= 1e-5 * np.abs(fd))
