"""GPU: the hand-written adjoints against the oracle (oracle/adjoint.py, itself
pinned by finite differences on the CPU) and central finite differences:
the per-facet-ti conduction step and its reverse sweep, the transpose
product of the compressed operator, the radiosity-solve backward and the
coupled radiosity + conduction misfit gradient with checkpointed segments."""
import numpy as np
import pytest
import scipy.sparse
import torch

from oracle import adjoint as A
from fluxpy_gb300 import adjoint as G
from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                  CompressedKernelMatrix, FormFactorOctreeBlock)
from fluxpy_gb300.thermal import PccThermalModel1D, setgrid

pytestmark = pytest.mark.gpu


def _pcc_case(N=300, seed=0):
    rng = np.random.default_rng(seed)
    z = np.concatenate([[0.0], setgrid(40, 1.0817, 1.0)])
    w = z.size
    T = rng.uniform(150, 300, (N, w))
    ti = np.linspace(55, 400, w)
    tif = np.tile(ti, (N, 1)) * rng.uniform(0.6, 1.4, (N, 1))
    rhoc = np.full(w, 1.2e6)
    em = rng.uniform(0.9, 0.98, N)
    Fg = np.full(N, 0.02)
    Qn = rng.uniform(0, 800, N)
    Qnp1 = rng.uniform(0, 800, N)
    Qn[:20], Qnp1[:20] = 1200.0, 0.0             # predictor-corrector redos
    Qn[20:30], Qnp1[20:30] = 0.0, 3000.0
    T[20:30] = 40.0
    return rng, z, T, ti, tif, rhoc, em, Fg, Qn, Qnp1


def _d(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def test_per_facet_ti_step_matches_oracle_bitwise():
    rng, z, T, ti, tif, rhoc, em, Fg, Qn, Qnp1 = _pcc_case()
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = G._step(_d(z), 3600.0, _d(Qn), _d(Qnp1), _d(T), _d(tif), z.size, _d(rhoc), _d(em),
                  _d(Fg), flags)
    ref, _, npass = A.pcc_q_forward(z, 3600.0, Qn, Qnp1, T, tif, rhoc, em, Fg, record=True)
    assert npass.max() >= 1
    assert np.array_equal(out.cpu().numpy(), ref)
    # one shared profile (row stride 0) equals the reference-layout kernel
    out0 = G._step(_d(z), 3600.0, _d(Qn), _d(Qnp1), _d(T), _d(ti), 0, _d(rhoc), _d(em), _d(Fg),
                   flags)
    m = PccThermalModel1D(z, T.copy(), ti, rhoc, em, Fg, Qn, T[:, 0].copy())
    m.step(3600.0, Qnp1)
    assert np.array_equal(out0.cpu().numpy(), m.T)
    assert int(flags.item()) == 0


def test_conduction_adjoint_matches_oracle():
    rng, z, T, ti, tif, rhoc, em, Fg, Qn, Qnp1 = _pcc_case()
    gT = rng.standard_normal(T.shape)
    ref = A.pcc_q_adjoint(z, 3600.0, Qn, Qnp1, T, tif, rhoc, em, Fg, gT)
    N, w = T.shape
    gem = torch.zeros(N, dtype=torch.float64, device="cuda")
    gti = torch.zeros((N, w), dtype=torch.float64, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    got = G._step_adjoint(_d(z), 3600.0, _d(Qn), _d(Qnp1), _d(T), _d(tif), w, _d(rhoc), _d(em),
                          _d(Fg), _d(gT), gem, gti, flags)
    got = [g.cpu().numpy() for g in got] + [gem.cpu().numpy(), gti.cpu().numpy()]
    for name, g, r in zip(["T", "Qn", "Qnp1", "emiss", "ti"], got, ref):
        err = np.abs(g - r).max() / np.abs(r).max()
        assert err < 1e-10, (name, err)
    # emiss and ti cotangents accumulate
    gem1 = gem.clone()
    G._step_adjoint(_d(z), 3600.0, _d(Qn), _d(Qnp1), _d(T), _d(tif), w, _d(rhoc), _d(em), _d(Fg),
                    _d(gT), gem, gti, flags)
    assert torch.equal(gem, 2 * gem1)
    assert int(flags.item()) == 0


def test_conduction_step_gradcheck():
    rng = np.random.default_rng(3)
    z = _d(np.concatenate([[0.0], setgrid(8, 1.2, 0.3)]))
    w = z.numel()
    N = 3
    T = _d(rng.uniform(180, 260, (N, w))).requires_grad_()
    Qn = _d(rng.uniform(100, 600, N)).requires_grad_()
    Qnp1 = _d(rng.uniform(100, 600, N)).requires_grad_()
    em = _d(rng.uniform(0.9, 0.98, N)).requires_grad_()
    ti = _d(rng.uniform(40, 120, (N, w))).requires_grad_()
    rhoc = _d(np.full(w, 1.2e6))
    Fg = _d(np.full(N, 0.02))

    def f(T_, a, b, e, t):
        return G.conduction_step(T_, a, b, e, t, z, rhoc, 1800.0, Fg)
    assert torch.autograd.gradcheck(f, (T, Qn, Qnp1, em, ti), eps=1e-6, atol=1e-6, rtol=1e-4)
    # per-facet ti uniform with depth: gradient summed over the layers
    ti1 = _d(rng.uniform(40, 120, N)).requires_grad_()
    assert torch.autograd.gradcheck(lambda t: f(T.detach(), Qn.detach(), Qnp1.detach(),
                                                em.detach(), t), (ti1,), eps=1e-6, atol=1e-6,
                                    rtol=1e-4)


@pytest.fixture(scope="module")
def op64():
    V, F = terrain.fbm_terrain(n=32, seed=4, n_craters=2)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=1024, dtype=np.float64,
                                    RootBlock=FormFactorOctreeBlock)
    assert FF.stats["lowrank_blocks"] > 0, FF.stats
    return sm, FF, FF.toarray()


def test_transpose_product_matches_dense(op64):
    sm, FF, Ad = op64
    rng = np.random.default_rng(1)
    y = rng.uniform(-1, 1, sm.num_faces)
    ref = Ad.T @ y
    got = FF.rmatvec(y)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-12
    Y = rng.uniform(0, 1, (sm.num_faces, 3))
    got2 = FF.rmatmat(Y)
    assert np.abs(got2 - Ad.T @ Y).max() / np.abs(Ad.T @ Y).max() < 1e-12
    # the FP32-stored copy of the same operator in FP64 arithmetic
    FF32 = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=1024, dtype=np.float32,
                                      RootBlock=FormFactorOctreeBlock)
    # (its toarray() rounds the low-rank entries to FP32, so the check is the
    # identity <F x, y> = <x, F^T y> with both products in FP64 arithmetic)
    yp = FF32.permute(_d(y))
    FTy = FF32.rmatvec_permuted(yp, "fp32-fp64")
    for _ in range(3):
        xp = FF32.permute(_d(rng.uniform(-1, 1, sm.num_faces)))
        Fx = FF32.matvec_permuted(xp, "fp32-fp64")
        lhs, rhs = torch.dot(Fx, yp).item(), torch.dot(xp, FTy).item()
        assert abs(lhs - rhs) <= 1e-13 * (xp.norm() * FTy.norm()).item(), (lhs, rhs)
    # CompressedKernelMatrix transpose products (compressed_form_factors.py:904-913)
    for place in ("right", "left"):
        Km = CompressedKernelMatrix(FF, 0.3, place)
        refk = y - (0.3 * (Ad.T @ y) if place == "right" else Ad.T @ (0.3 * y))
        assert np.abs(Km.rmatvec(y) - refk).max() / np.abs(refk).max() < 1e-12
    FF.check_device_flags()


def test_radiosity_solve_backward_matches_dense(op64):
    sm, FF, Ad = op64
    N = sm.num_faces
    rng = np.random.default_rng(2)
    dirs = terrain.random_sun_directions(2, seed=2)
    E = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float64).contiguous()
    E.requires_grad_()
    rho = _d(rng.uniform(0.07, 0.2, N)).requires_grad_()
    W = _d(rng.standard_normal((N, 2)))
    B = G.radiosity_solve(FF, E, rho)
    (B * W).sum().backward()
    En = E.detach().cpu().numpy()
    rn = rho.detach().cpu().numpy()
    M = np.eye(N) - Ad * rn[None, :]
    Bref = np.linalg.solve(M, En)
    lam = np.linalg.solve(M.T, W.cpu().numpy())
    grho = np.sum(Bref * (Ad.T @ lam), axis=1)
    assert np.abs(B.detach().cpu().numpy() - Bref).max() / np.abs(Bref).max() < 1e-11
    assert np.abs(E.grad.cpu().numpy() - lam).max() / np.abs(lam).max() < 1e-11
    assert np.abs(rho.grad.cpu().numpy() - grho).max() / np.abs(grho).max() < 1e-10
    # scalar albedo: its gradient is the sum over facets
    r0 = torch.tensor(0.12, dtype=torch.float64, device="cuda", requires_grad=True)
    (G.radiosity_solve(FF, E.detach(), r0) * W).sum().backward()
    M0 = np.eye(N) - 0.12 * Ad
    B0 = np.linalg.solve(M0, En)
    lam0 = np.linalg.solve(M0.T, W.cpu().numpy())
    g0 = np.sum(B0 * (Ad.T @ lam0))
    assert abs(r0.grad.item() - g0) / abs(g0) < 1e-10


def _misfit_case(sm, S=8, seed=4):
    N = sm.num_faces
    rng = np.random.default_rng(seed)
    dirs = terrain.random_sun_directions(S + 1, seed=2, elev=(5, 40))
    E = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float64)
    z = np.concatenate([[0.0], setgrid(20, 1.1, 0.5)])
    w = z.size
    return dict(E=E.cpu().numpy(), z=z, rhoc=np.full(w, 1.2e6), dt=3600.0,
                T0=np.full((N, w), 200.0), Fgeotherm=np.full(N, 0.02),
                Tobs=rng.uniform(150, 300, (N, S))), dict(
        rho=rng.uniform(0.07, 0.2, N), emiss=rng.uniform(0.9, 0.98, N),
        ti=rng.uniform(40, 120, N))


def test_thermal_misfit_gradient_matches_oracle_and_fd(op64):
    sm, FF, Ad = op64
    case, par = _misfit_case(sm)
    m = G.ThermalMisfit(FF, case["E"], case["z"], case["rhoc"], case["dt"], case["T0"],
                        case["Fgeotherm"], case["Tobs"], checkpoint_every=3, tol=1e-14)
    L, grho, gem, gti = m.value_and_grad(par["rho"], par["emiss"], par["ti"])
    Lo, grho_o, gem_o, gti_o = A.coupled_gradient(Ad, case["E"], par["rho"], par["emiss"],
                                                  par["ti"], case["z"], case["rhoc"], case["dt"],
                                                  case["T0"], case["Fgeotherm"], case["Tobs"])
    assert abs(L.item() - Lo) / Lo < 1e-11
    for g, r in ((grho, grho_o), (gem, gem_o), (gti, gti_o)):
        g = g.cpu().numpy()
        assert np.abs(g - r).max() / np.abs(r).max() < 1e-9
    # central finite differences of the GPU forward model (the 1e-4 bar)
    rng = np.random.default_rng(7)
    grads = dict(rho=grho.cpu().numpy(), emiss=gem.cpu().numpy(), ti=gti.cpu().numpy())
    for key in ("rho", "emiss", "ti"):
        for i in rng.choice(sm.num_faces, 4, replace=False):
            x = par[key]
            h = 1e-5 * x[i]
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            Lp = m.value(**{**par, key: xp}).item()
            Lm = m.value(**{**par, key: xm}).item()
            fd = (Lp - Lm) / (2 * h)
            assert abs(fd - grads[key][i]) <= 1e-4 * abs(fd), (key, i, fd, grads[key][i])
    # the same gradient through torch.autograd, and with a sparse operator
    t = {k: _d(v).requires_grad_() for k, v in par.items()}
    G.thermal_misfit(m, t["rho"], t["emiss"], t["ti"]).backward()
    # (the transposed operator's products are deterministic: bit-identical)
    assert torch.equal(t["rho"].grad, grho)
    assert torch.equal(t["ti"].grad, gti)
    ms = G.ThermalMisfit(scipy.sparse.csr_matrix(Ad), case["E"], case["z"], case["rhoc"],
                         case["dt"], case["T0"], case["Fgeotherm"], case["Tobs"],
                         checkpoint_every=25, tol=1e-14)
    Ls, grho_s, gem_s, gti_s = ms.value_and_grad(par["rho"], par["emiss"], par["ti"])
    assert abs(Ls.item() - Lo) / Lo < 1e-11
    assert np.abs(gem_s.cpu().numpy() - gem_o).max() / np.abs(gem_o).max() < 1e-9


@pytest.fixture(scope="module")
def op32():
    V, F = terrain.fbm_terrain(n=32, seed=4, n_craters=2)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=1024, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    N = sm.num_faces
    # the stored operator in cluster order, FP64 arithmetic, column by column
    eye = torch.eye(N, dtype=torch.float64, device="cuda")
    D = torch.stack([FF.matvec_permuted(eye[:, c].contiguous(), "fp32-fp64") for c in range(N)], 1)
    return sm, FF, D


def test_transposed_operator_products(op32):
    """F^T through the transposed copy of the operator, K columns at once,
    in every precision, against the transpose of the stored operator."""
    sm, FF, D = op32
    N = sm.num_faces
    T = FF.transposed()
    assert T is FF.transposed()                       # cached
    rng = np.random.default_rng(5)
    Y = _d(rng.uniform(-1, 1, (N, 40)))
    ref = D.T @ Y
    scale = ref.abs().max().item()
    got64 = T.matmat_permuted(Y, "fp32-fp64")
    assert (got64 - ref).abs().max().item() <= 1e-13 * scale
    # K = 1 products of the transpose are the same columns
    assert torch.allclose(FF.rmatvec_permuted(Y[:, 3].contiguous()), got64[:, 3], rtol=0,
                          atol=1e-14 * scale)
    got32 = T.matmat_permuted(Y.float(), "fp32").double()
    assert (got32 - ref).abs().max().item() <= 1e-5 * scale
    got16 = T.matmat_permuted(Y.float(), "bf16").double()
    assert (got16 - ref).abs().max().item() <= 3e-2 * scale
    # the forward K-column FP64-arithmetic product agrees with the dense one too
    fwd = FF.matmat_permuted(Y, "fp32-fp64")
    assert (fwd - D @ Y).abs().max().item() <= 1e-13 * (D @ Y).abs().max().item()


def test_refined_solves_match_dense(op32):
    """Many columns solved by FP32 sweeps with FP64 residuals (the
    adjoint's forward and transposed solves) against dense FP64 solves."""
    sm, FF, D = op32
    N = sm.num_faces
    ops = G._ops(FF, torch.device("cuda"))
    assert ops.batched
    rng = np.random.default_rng(6)
    E = _d(rng.uniform(0, 1000, (N, 24)))
    rho = _d(rng.uniform(0.07, 0.2, N))
    B = G.solve_right(ops, E, rho, tol=1e-13)
    lam = G.solve_right_T(ops, E, rho, tol=1e-13)
    perm = FF._perm_d
    Ep = E[perm]
    rp = rho[perm]
    I = torch.eye(N, dtype=torch.float64, device="cuda")
    Bd = torch.linalg.solve(I - D * rp[None, :], Ep)
    Ld = torch.linalg.solve(I - rp[:, None] * D.T, Ep)
    assert (B[perm] - Bd).abs().max().item() <= 1e-11 * Bd.abs().max().item()
    assert (lam[perm] - Ld).abs().max().item() <= 1e-11 * Ld.abs().max().item()


def test_gradient_at_10k_facets_matches_dense_fp64_oracle():
    """The coupled misfit's gradient on a 9,800-facet fBm terrain against
    the oracle's dense FP64 gradient: through the exact form factors (the
    adjoint's own accuracy) and through the compressed FP32-stored operator
    with refined many-column solves (the compression's share)."""
    from fluxpy_gb300.form_factors import get_form_factor_matrix
    V, F = terrain.fbm_terrain(n=71, seed=4)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    assert 9000 < sm.num_faces < 11000
    Fx = get_form_factor_matrix(sm)
    case, par = _misfit_case(sm, S=6, seed=9)
    Lo, grho_o, gem_o, gti_o = A.coupled_gradient(Fx.toarray(), case["E"], par["rho"],
                                                  par["emiss"], par["ti"], case["z"], case["rhoc"],
                                                  case["dt"], case["T0"], case["Fgeotherm"],
                                                  case["Tobs"])
    args = (case["E"], case["z"], case["rhoc"], case["dt"], case["T0"], case["Fgeotherm"],
            case["Tobs"])
    m = G.ThermalMisfit(Fx, *args, checkpoint_every=4, tol=1e-14)
    L, grho, gem, gti = m.value_and_grad(par["rho"], par["emiss"], par["ti"])
    assert abs(L.item() - Lo) / Lo < 1e-11
    for g, r in ((grho, grho_o), (gem, gem_o), (gti, gti_o)):
        assert np.abs(g.cpu().numpy() - r).max() / np.abs(r).max() < 1e-9
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    mc = G.ThermalMisfit(FF, *args, checkpoint_every=4, tol=1e-13)
    assert mc.ops.batched
    Lc, grho_c, gem_c, gti_c = mc.value_and_grad(par["rho"], par["emiss"], par["ti"])
    assert abs(Lc.item() - Lo) / Lo < 1e-5
    for g, r in ((grho_c, grho_o), (gem_c, gem_o), (gti_c, gti_o)):
        assert np.abs(g.cpu().numpy() - r).max() / np.abs(r).max() < 1e-3
