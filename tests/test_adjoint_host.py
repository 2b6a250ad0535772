"""CPU: the host logic of fluxpy_gb300.adjoint (checkpointed reverse sweep,
transposed solves, autograd plumbing, ti shapes) with its device calls
replaced by the oracle's CPU restatements (oracle/adjoint.py) and a dense
form-factor matrix.  The device kernels themselves are checked against the
same oracle in test_gpu_adjoint.py."""
import numpy as np
import pytest
import torch

from oracle import adjoint as A
from oracle import vis
from fluxpy_gb300 import _lib, terrain
from fluxpy_gb300 import adjoint as G
from fluxpy_gb300.thermal import setgrid


class _DenseOps:
    batched = False   # plain Jacobi solves (no refinement)

    def __init__(self, Ad):
        self.M = torch.as_tensor(Ad)
        self.N = Ad.shape[0]

    def F(self, x):
        return self.M @ x

    def FT(self, y):
        return self.M.T @ y


@pytest.fixture
def cpu_device_calls(monkeypatch):
    def step(z, dt, Qn, Qnp1, T, ti, ld, rhoc, em, Fg, flags):
        tin = ti.numpy() if ld else np.broadcast_to(ti.numpy(), T.shape)
        return torch.as_tensor(A.pcc_q_forward(z.numpy(), dt, Qn.numpy(), Qnp1.numpy(),
                                               T.numpy(), tin, rhoc.numpy(), em.numpy(),
                                               Fg.numpy()))

    def step_adjoint(z, dt, Qn, Qnp1, T, ti, ld, rhoc, em, Fg, gT, gem, gti, flags):
        tin = ti.numpy() if ld else np.broadcast_to(ti.numpy(), T.shape)
        a, b, c, d, e = A.pcc_q_adjoint(z.numpy(), dt, Qn.numpy(), Qnp1.numpy(), T.numpy(), tin,
                                        rhoc.numpy(), em.numpy(), Fg.numpy(), gT.numpy())
        gem += torch.as_tensor(d)
        gti += torch.as_tensor(e)
        return torch.as_tensor(a), torch.as_tensor(b), torch.as_tensor(c)

    monkeypatch.setattr(G, "_step", step)
    monkeypatch.setattr(G, "_step_adjoint", step_adjoint)
    monkeypatch.setattr(G, "_raise_flags", lambda flags: None)
    monkeypatch.setattr(_lib, "require_cuda", lambda: torch.device("cpu"))


def _case():
    V, F = terrain.fbm_terrain(n=10, seed=4, n_craters=1)
    P, Nn, Ar = vis.geometry(V, F)
    Ad = vis.Scene(V, F).ff_csr(P, Nn, Ar).toarray()
    N = Ad.shape[0]
    rng = np.random.default_rng(4)
    S = 8
    dirs = terrain.random_sun_directions(S + 1, seed=2, elev=(5, 40))
    E = np.stack([1365 * np.maximum(0, Nn @ d) for d in dirs], 1)
    z = np.concatenate([[0.0], setgrid(20, 1.1, 0.5)])
    case = dict(E=E, z=z, rhoc=np.full(z.size, 1.2e6), dt=3600.0, T0=np.full((N, z.size), 200.0),
                Fgeotherm=np.full(N, 0.02), Tobs=rng.uniform(150, 300, (N, S)))
    par = dict(rho=rng.uniform(0.07, 0.2, N), emiss=rng.uniform(0.9, 0.98, N),
               ti=rng.uniform(40, 120, N))
    return Ad, case, par


@pytest.mark.parametrize("every", [1, 3, 8, 25])
def test_checkpointed_sweep_equals_oracle_gradient(cpu_device_calls, monkeypatch, every):
    Ad, case, par = _case()
    monkeypatch.setattr(G, "_ops", lambda FF, dev: _DenseOps(Ad))
    m = G.ThermalMisfit(Ad, case["E"], case["z"], case["rhoc"], case["dt"], case["T0"],
                        case["Fgeotherm"], case["Tobs"], checkpoint_every=every, tol=1e-14)
    L, grho, gem, gti = m.value_and_grad(par["rho"], par["emiss"], par["ti"])
    Lo, grho_o, gem_o, gti_o = A.coupled_gradient(Ad, case["E"], par["rho"], par["emiss"],
                                                  par["ti"], case["z"], case["rhoc"], case["dt"],
                                                  case["T0"], case["Fgeotherm"], case["Tobs"])
    assert abs(L.item() - Lo) <= 1e-12 * Lo
    for g, r in ((grho, grho_o), (gem, gem_o), (gti, gti_o)):
        assert np.abs(g.numpy() - r).max() <= 1e-10 * np.abs(r).max()
    assert abs(m.value(**par).item() - Lo) <= 1e-12 * Lo
    Ts = m.surface_temperatures(**par)
    assert Ts.shape == (Ad.shape[0], case["Tobs"].shape[1])
    # through torch.autograd
    t = {k: torch.tensor(v, requires_grad=True) for k, v in par.items()}
    G.thermal_misfit(m, t["rho"], t["emiss"], t["ti"]).backward()
    assert torch.allclose(t["ti"].grad, gti, rtol=1e-12, atol=0)


def test_radiosity_solve_backward_dense(cpu_device_calls, monkeypatch):
    Ad, case, par = _case()
    monkeypatch.setattr(G, "_ops", lambda FF, dev: _DenseOps(Ad))
    N = Ad.shape[0]
    rng = np.random.default_rng(5)
    E = torch.tensor(case["E"][:, :3].copy(), requires_grad=True)
    rho = torch.tensor(par["rho"], requires_grad=True)
    W = torch.as_tensor(rng.standard_normal((N, 3)))
    B = G.RadiositySolve.apply(E, rho, None, 1e-14, 1000)
    (B * W).sum().backward()
    M = np.eye(N) - Ad * par["rho"][None, :]
    lam = np.linalg.solve(M.T, W.numpy())
    Bref = np.linalg.solve(M, case["E"][:, :3])
    assert np.abs(B.detach().numpy() - Bref).max() <= 1e-12 * np.abs(Bref).max()
    assert np.abs(E.grad.numpy() - lam).max() <= 1e-12 * np.abs(lam).max()
    grho = np.sum(Bref * (Ad.T @ lam), axis=1)
    assert np.abs(rho.grad.numpy() - grho).max() <= 1e-10 * np.abs(grho).max()


@pytest.mark.parametrize("ti_shape", ["layers", "facets", "full"])
def test_conduction_step_gradcheck_host(cpu_device_calls, ti_shape):
    rng = np.random.default_rng(3)
    z = torch.tensor(np.concatenate([[0.0], setgrid(8, 1.2, 0.3)]))
    w = z.numel()
    N = 3
    T = torch.tensor(rng.uniform(180, 260, (N, w)), requires_grad=True)
    Qn = torch.tensor(rng.uniform(100, 600, N), requires_grad=True)
    Qnp1 = torch.tensor(rng.uniform(100, 600, N), requires_grad=True)
    em = torch.tensor(rng.uniform(0.9, 0.98, N), requires_grad=True)
    shape = {"layers": (w,), "facets": (N,), "full": (N, w)}[ti_shape]
    ti = torch.tensor(rng.uniform(40, 120, shape), requires_grad=True)
    rhoc = torch.tensor(np.full(w, 1.2e6))
    Fg = torch.tensor(np.full(N, 0.02))

    def f(T_, a, b, e, t):
        return G.conduction_step(T_, a, b, e, t, z, rhoc, 1800.0, Fg)
    assert torch.autograd.gradcheck(f, (T, Qn, Qnp1, em, ti), eps=1e-6, atol=1e-6, rtol=1e-4)


def test_input_checks(cpu_device_calls, monkeypatch):
    Ad, case, par = _case()
    monkeypatch.setattr(G, "_ops", lambda FF, dev: _DenseOps(Ad))
    with pytest.raises(ValueError):
        G.ThermalMisfit(Ad, case["E"], case["z"], case["rhoc"], case["dt"], case["T0"],
                        case["Fgeotherm"], case["Tobs"][:, :-1])
    with pytest.raises(ValueError):
        G.ThermalMisfit(Ad, case["E"][:, :1], case["z"], case["rhoc"], case["dt"], case["T0"],
                        case["Fgeotherm"], case["Tobs"][:, :0])
    m = G.ThermalMisfit(Ad, case["E"], case["z"], case["rhoc"], case["dt"], case["T0"],
                        case["Fgeotherm"], case["Tobs"])
    with pytest.raises(ValueError):
        m.value(par["rho"][:-1], par["emiss"], par["ti"])
    with pytest.raises(ValueError):
        m.value(par["rho"], par["emiss"], np.ones((3, 3)))
