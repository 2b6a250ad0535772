"""GPU: compressed form-factor operator (block structure, exact leaves, ACA
low-rank blocks), its matvec kernels, and the radiosity / steady-state
solves, against the oracle's exact form factors and the reference's own
solves (tests/golden/ffref.npz)."""
import itertools as it

import numpy as np
import pytest
import scipy.sparse
import torch

from oracle import vis
from tests.conftest import GOLDEN
from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (
    CompressedFormFactorMatrix, CompressedKernelMatrix, FormFactorDenseBlock,
    FormFactorOctreeBlock, FormFactorQuadtreeBlock, FormFactorZeroBlock)
from fluxpy_gb300.form_factors import get_form_factor_matrix
from fluxpy_gb300.model import compute_steady_state_temp
from fluxpy_gb300.solve import solve_radiosity, solve_radiosity_batched

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ffref():
    return np.load(GOLDEN / "ffref.npz")


@pytest.fixture(scope="module")
def spheres():
    return np.load(GOLDEN / "spheres.npz")


@pytest.mark.parametrize("cls", [gshape.EmbreeTrimeshShapeModel, gshape.CgalTrimeshShapeModel])
@pytest.mark.parametrize("name", ["icosa_sphere", "icosa_sphere_5"])
def test_max_depth_1_for_stretched_sphere(spheres, cls, name):
    # tests/test_compressed_form_factors.py:25-76 of the reference
    V, F = spheres[f"{name}_V"].copy(), spheres[f"{name}_F"]
    V *= np.random.default_rng(3).random(3)
    sm = cls(V, F)
    outward = (sm.P * sm.N).sum(1) > 0
    sm.N[outward] *= -1
    FF = CompressedFormFactorMatrix(sm, tol=0, max_depth=1, force_max_depth=True,
                                    RootBlock=FormFactorOctreeBlock)
    FF_gt = get_form_factor_matrix(sm).toarray()
    assert FF.depth == 1
    for i, j in it.product(range(8), repeat=2):
        block = FF._root._blocks[i, j]
        assert block.is_leaf
        assert isinstance(block, (FormFactorDenseBlock, FormFactorZeroBlock))
        I = FF._root._row_block_inds[i]
        J = FF._root._col_block_inds[j]
        if I.size and J.size:
            assert isinstance(block, FormFactorDenseBlock)
            assert (block._mat == FF_gt[I, :][:, J]).all()
    E = np.random.default_rng(4).standard_normal(sm.num_faces)
    B, B_gt = FF @ E, FF_gt @ E
    assert abs(B - B_gt).max() / abs(B_gt).max() < 1e-14


def test_octree_sphere_matches_reference_golden(ffref):
    sm = gshape.EmbreeTrimeshShapeModel(ffref["octsphere_V"], ffref["octsphere_F"],
                                        N=ffref["octsphere_N"].copy())
    FF = CompressedFormFactorMatrix(sm, tol=0, max_depth=1, force_max_depth=True,
                                    RootBlock=FormFactorOctreeBlock)
    assert [len(r) for r in FF._root._row_block_inds] == list(ffref["octsphere_rows"])
    types = [type(b).__name__ for b in FF._root._blocks.ravel()]
    assert types == list(ffref["octsphere_types"])
    y = FF @ ffref["octsphere_x"]
    assert np.allclose(y, ffref["octsphere_y"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("max_depth", [1, 2, 3])
def test_quadtree_crater_exact(ffref, max_depth):
    # tests/test_compressed_form_factors.py:152-190 (tol = 0): the product
    # equals the uncompressed matrix's to round-off
    sm = gshape.EmbreeTrimeshShapeModel(ffref["crater_V"], ffref["crater_F"])
    FF = CompressedFormFactorMatrix(sm, tol=0, max_depth=max_depth, min_size=4096,
                                    RootBlock=FormFactorQuadtreeBlock)
    FF_gt = get_form_factor_matrix(sm)
    E = ffref["crater_E"]
    B, B_gt = FF @ E, FF_gt @ E
    assert abs(B - B_gt).max() / abs(B_gt).max() < np.finfo(np.float64).resolution
    # and the reference's own compressed product on the same matrix
    y_ref = ffref[f"crater_quad{max_depth}_y"]
    assert np.allclose(B, y_ref, rtol=1e-9, atol=1e-12 * abs(y_ref).max())


def _terrain_case(n=64, seed=5):
    V, F = terrain.fbm_terrain(n=n, seed=seed, n_craters=6)
    return gshape.EmbreeTrimeshShapeModel(V, F)


def test_compressed_lowrank_error_vs_exact():
    sm = _terrain_case(64)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096,
                                    RootBlock=FormFactorOctreeBlock)
    st = FF.stats
    assert st["lowrank_blocks"] > 0, st
    Fx = get_form_factor_matrix(sm)
    rng = np.random.default_rng(0)
    for _ in range(3):
        x = rng.uniform(0, 1, sm.num_faces)
        y = FF @ x
        y_gt = Fx @ x
        err = abs(y - y_gt).max() / abs(y_gt).max()
        assert err < 1e-5, (err, st)
    # FP32 and BF16 device products against the FP64 one
    X = torch.as_tensor(rng.uniform(0, 1, (sm.num_faces, 64)), device="cuda")
    Xp = FF.permute(X)
    Y64 = FF.matmat_permuted(Xp[:, :4].contiguous(), "fp64")
    Y32 = FF.matmat_permuted(Xp, "fp32")
    Yb = FF.matmat_permuted(Xp, "bf16")
    y1 = FF.matvec_permuted(Xp[:, 0].contiguous(), "fp32")
    ref = Y64.abs().max().item()
    assert (Y32[:, :4].double() - Y64).abs().max().item() / ref < 1e-5
    assert (y1.double() - Y64[:, 0]).abs().max().item() / ref < 1e-5
    assert (Yb[:, :4].double() - Y64).abs().max().item() / ref < 2e-2


def test_batched_steady_state_matches_reference_golden(ffref):
    """compute_steady_state_temp with method='batched-bf16' (BF16+refine
    solves, split-BF16 tensor-core infrared product) on the compressed
    operator of the crater, against the reference's own T for three sun
    directions (tests/golden/ffref.npz)."""
    sm = gshape.EmbreeTrimeshShapeModel(ffref["crater_V"], ffref["crater_F"])
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=1024, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    E2 = ffref["crater_E2"]
    T2 = compute_steady_state_temp(FF, E2, 0.12, 0.95, method="batched-bf16")
    assert T2.shape == ffref["crater_T2"].shape
    # (measured on GB300: 1.6e-4 K; the solves stop at 1e-5 relative)
    assert np.max(np.abs(T2 - ffref["crater_T2"])) < 1e-3
    # the same with the FP32 batched method (CUDA-core infrared product)
    T3 = compute_steady_state_temp(FF, E2, 0.12, 0.95, method="batched-fp32")
    assert np.max(np.abs(T3 - ffref["crater_T2"])) < 1e-3
    # an operator without low-rank blocks (tol = 0: no Z rows) through the
    # same tensor-core path
    FF0 = CompressedFormFactorMatrix(sm, tol=0, min_size=1024, dtype=np.float32,
                                     RootBlock=FormFactorOctreeBlock)
    assert FF0._num_zrows == 0
    T0 = compute_steady_state_temp(FF0, E2, 0.12, 0.95, method="batched-bf16")
    assert np.max(np.abs(T0 - ffref["crater_T2"])) < 1e-3


def test_solve_matches_reference_golden(ffref):
    sm = gshape.EmbreeTrimeshShapeModel(ffref["crater_V"], ffref["crater_F"])
    FF = get_form_factor_matrix(sm)
    E = ffref["crater_E"]
    B, niter = solve_radiosity(FF, E, 0.12, "right", "jacobi")
    assert niter == int(ffref["crater_niter"])
    assert np.allclose(B, ffref["crater_B"], rtol=1e-9, atol=1e-9)
    T = compute_steady_state_temp(FF, E, 0.12, 0.95)
    assert np.max(np.abs(T - ffref["crater_T"])) < 1e-6
    B2, n2 = solve_radiosity(FF, ffref["crater_E2"], 0.12, "right", "jacobi")
    assert n2 == int(ffref["crater_niter2"])
    assert np.allclose(B2, ffref["crater_B2"], rtol=1e-9, atol=1e-9)
    T2 = compute_steady_state_temp(FF, ffref["crater_E2"], 0.12, 0.95)
    assert np.max(np.abs(T2 - ffref["crater_T2"])) < 1e-6
    # left placement and CG agree with the right-placement solution
    Bl, _ = solve_radiosity(FF, E, 0.12, "left", "jacobi")
    Bc, _ = solve_radiosity(FF, E, 0.12, "left", "cg")
    assert np.allclose(Bl, Bc, rtol=1e-8, atol=1e-8)
    with pytest.raises(NotImplementedError):
        solve_radiosity(FF, E, 0.12, "right", "cg")


def test_solve_per_facet_albedo_matches_oracle(ffref):
    """solve_radiosity with one albedo per facet (numpy array), right and
    left placement, on the crater's exact form factors: the oracle's Jacobi
    iteration count and solution (src/flux/solve.py:36-45 multiplies
    rho * B elementwise)."""
    from oracle import solve as osolve
    sm = gshape.EmbreeTrimeshShapeModel(ffref["crater_V"], ffref["crater_F"])
    FF = get_form_factor_matrix(sm)
    E = ffref["crater_E"]
    rho = np.random.default_rng(8).uniform(0.05, 0.4, sm.num_faces)
    for placement in ("right", "left"):
        B, niter = solve_radiosity(FF, E, rho, placement, "jacobi")
        Bo, no = osolve.solve_radiosity(FF, E, rho, placement)
        # (the stopping test sits at FP64 resolution: a product summed in
        # another order may end one iteration earlier or later)
        assert abs(niter - no) <= 1
        assert np.allclose(B, Bo, rtol=1e-9, atol=1e-9 * abs(Bo).max())
    # the compressed operator (tol = 0) through the same path
    FFc = CompressedFormFactorMatrix(sm, tol=0, min_size=4096)
    Bc, nc = solve_radiosity(FFc, E, rho)
    Bo, no = osolve.solve_radiosity(FF, E, rho)
    assert abs(nc - no) <= 1 and np.allclose(Bc, Bo, rtol=1e-9, atol=1e-9 * abs(Bo).max())
    # and the steady-state temperature of one direction (model.py:8-42
    # takes rho per facet through the same solve)
    T = compute_steady_state_temp(FF, E, rho, 0.95)
    To = osolve.steady_state_temp(FF, E, rho, 0.95)
    assert np.max(np.abs(T - To)) < 1e-6


def test_solve_with_compressed_operator_and_kernel_matrix(ffref):
    sm = gshape.EmbreeTrimeshShapeModel(ffref["crater_V"], ffref["crater_F"])
    FF = CompressedFormFactorMatrix(sm, tol=0, min_size=4096)
    E = ffref["crater_E"]
    B, niter = solve_radiosity(FF, E, 0.12)
    assert niter == int(ffref["crater_niter"])
    assert np.allclose(B, ffref["crater_B"], rtol=1e-9, atol=1e-9)
    Kop = CompressedKernelMatrix(FF, 0.12)
    r = Kop @ B - E  # (I - rho F) B - E, small at convergence
    assert abs(r).max() <= 1e-9 * abs(E).max()


def test_batched_solvers_reach_rtol():
    sm = _terrain_case(48, seed=9)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    dirs = terrain.random_sun_directions(64, seed=2)
    E = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    assert E.shape == (sm.num_faces, 64)
    cases = [("fp32", "tc", "fp32", True, 2e-5), ("bf16-refine", "tc", "split-bf16", True, 1e-5),
             ("bf16-refine", "tc", "split-bf16", False, 1e-5),
             ("bf16-refine", "tc", "fp32", True, 1e-5), ("bf16-refine", "mma", "fp32", True, 1e-5)]
    for prec, eng, res, incr, bound in cases:
        st = {}
        B = solve_radiosity_batched(FF, E, 0.12, rtol=1e-5, precision=prec, stats=st,
                                    engine=eng, residual=res, incremental=incr)
        # residual with the operator in FP64 arithmetic; the plain Jacobi
        # path stops on its update size (as the reference does), the
        # refinement on the residual itself
        Bp = FF.permute(B.double())
        FBp = FF.matmat_permuted(Bp[:, :8].contiguous() * 0.12, "fp64")
        Ep = FF.permute(E.double())[:, :8]
        R = Ep - (Bp[:, :8] - FBp)
        rel = (R.abs().amax(0) / Ep.abs().amax(0).clamp_min(1e-30)).max().item()
        assert rel <= bound, (prec, eng, res, incr, rel, st)


def test_batched_solve_edge_cases():
    """Batched solves with a per-facet albedo, a column count that is not a
    multiple of 8 (padded internally), a zero column (a sun below the
    horizon) and columns solved in chunks: every column reaches rtol in FP64
    arithmetic, the zero column stays exactly zero, and the chunked solve
    agrees with the one-block solve."""
    sm = _terrain_case(32, seed=7)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    dirs = terrain.random_sun_directions(20, seed=4)
    E20 = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    E = torch.cat([E20[:, :9], torch.zeros_like(E20[:, :1]), E20[:, 9:]], 1).contiguous()
    assert E.shape[1] == 21
    rho = np.random.default_rng(11).uniform(0.05, 0.3, sm.num_faces)
    rho_p = FF.permute(torch.as_tensor(rho, device=E.device)).reshape(-1, 1)
    Ep = FF.permute(E.double())
    emax = Ep.abs().amax(0)
    nz = emax > 0

    def rel_residual(B):
        Bp = FF.permute(B.double())
        R = Ep - (Bp - FF.matmat_permuted((rho_p * Bp).contiguous(), "fp64"))
        return (R.abs().amax(0)[nz] / emax[nz]).max().item()

    for prec, bound in (("bf16-refine", 1e-5), ("fp32", 2e-5)):
        st, stc = {}, {}
        B = solve_radiosity_batched(FF, E, rho, rtol=1e-5, precision=prec, stats=st)
        assert B.shape == E.shape and B.dtype == torch.float32
        assert rel_residual(B) <= bound, (prec, st)
        assert torch.count_nonzero(B[:, 9]).item() == 0
        Bc = solve_radiosity_batched(FF, E, rho, rtol=1e-5, precision=prec, stats=stc, chunk=8)
        assert stc["chunks"] == 3
        assert rel_residual(Bc) <= bound, (prec, stc)
        assert torch.count_nonzero(Bc[:, 9]).item() == 0
        diff = ((Bc - B).abs().amax(0)[nz] / B.abs().amax(0)[nz]).max().item()
        assert diff <= 4 * bound, (prec, diff)
        if prec == "bf16-refine":
            B_bf16 = B
    # more columns than one block takes (8,192): equal blocks of 4,104
    Ew = E.repeat(1, 391)[:, :8200].contiguous()
    stw = {}
    Bw = solve_radiosity_batched(FF, Ew, rho, rtol=1e-5, stats=stw)
    assert stw["chunks"] == 2 and Bw.shape == Ew.shape
    assert torch.count_nonzero(Bw[:, 9::21]).item() == 0
    Bw3 = Bw[:, :8190].reshape(-1, 390, 21)
    den = B_bf16.abs().amax(0).clamp_min(1e-30)
    diff = ((Bw3 - B_bf16[:, None, :]).abs().amax(0) / den).amax(0)[nz].max().item()
    assert diff <= 4e-5, diff
    # no columns
    st0 = {}
    B0 = solve_radiosity_batched(FF, E[:, :0], rho, stats=st0)
    assert B0.shape == (sm.num_faces, 0) and st0["outer"] == 0


def test_public_batched_solve_host_buffers():
    """solve_radiosity(..., method='batched-bf16' / 'batched-fp32') with host
    inputs: numpy in, numpy out; a pinned tensor in, a pinned tensor out;
    out= receives B; all equal to the device-resident batched solve."""
    sm = _terrain_case(32, seed=5)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    dirs = terrain.random_sun_directions(16, seed=3)
    E = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    for method, prec in (("batched-bf16", "bf16-refine"), ("batched-fp32", "fp32")):
        Bd = solve_radiosity_batched(FF, E, 0.12, rtol=1e-5, precision=prec).cpu()
        Bn, niter = solve_radiosity(FF, E.cpu().numpy(), 0.12, method=method)
        assert isinstance(Bn, np.ndarray) and niter >= 1
        assert np.array_equal(Bn, Bd.numpy())
        Ep = torch.empty(E.shape, dtype=torch.float32, pin_memory=True)
        Ep.copy_(E.cpu())
        Bt, _ = solve_radiosity(FF, Ep, 0.12, method=method)
        assert isinstance(Bt, torch.Tensor) and not Bt.is_cuda and Bt.is_pinned()
        assert torch.equal(Bt, Bd)
        out = torch.full(E.shape, float("nan"), pin_memory=True)
        Bo, _ = solve_radiosity(FF, Ep, 0.12, method=method, out=out)
        assert Bo is out and torch.equal(out, Bd)
        outn = np.full(tuple(E.shape), np.nan, np.float32)
        Bo, _ = solve_radiosity(FF, E.cpu().numpy(), 0.12, method=method, out=outn)
        assert Bo is outn and np.array_equal(outn, Bd.numpy())
        # one column as a vector
        b, _ = solve_radiosity(FF, E[:, 3].cpu().numpy(), 0.12, method=method)
        assert b.shape == (sm.num_faces,)
    # the side-stream copy of each candidate B: the host buffer and the
    # returned B equal a solve without it, also when some copies are of
    # candidates that the next check rejects (one first sweep, no correction
    # sweeps and rho = 0.5: more outer iterations)
    copies = []
    for inner0, inner, rho in ((2, 1, 0.12), (1, 0, 0.5)):
        st0, st1 = {}, {}
        Bd = solve_radiosity_batched(FF, E, rho, inner0=inner0, inner=inner, stats=st0)
        hb = torch.full(E.shape, float("nan"), pin_memory=True)
        B1 = solve_radiosity_batched(FF, E, rho, inner0=inner0, inner=inner, stats=st1,
                                     host_out=hb)
        torch.cuda.synchronize()
        assert st1["outer"] == st0["outer"] and torch.equal(B1, Bd)
        # a copy is offered after each correction; the one of the accepted B
        # fills the buffer (none when the first residual check accepts)
        assert st1["host_out_copies"] == st1["outer"] - 1
        assert st1["host_out_overlapped"] == (st1["outer"] >= 2)
        assert torch.equal(hb, Bd.cpu())
        copies.append(st1["host_out_copies"])
    assert max(copies) >= 2
    # paths without the side-stream copy (FP32, column blocks) fill it after
    # the solve
    for kw in ({"precision": "fp32"}, {"chunk": 8}):
        st2 = {}
        Bd = solve_radiosity_batched(FF, E, 0.12, **kw)
        hb = torch.full(E.shape, float("nan"), pin_memory=True)
        B2 = solve_radiosity_batched(FF, E, 0.12, stats=st2, host_out=hb, **kw)
        assert not st2.get("host_out_overlapped") and torch.equal(B2, Bd)
        assert torch.equal(hb, Bd.cpu())
    with pytest.raises(ValueError, match="return_permuted"):
        solve_radiosity_batched(FF, E, 0.12, return_permuted=True,
                                host_out=torch.empty(E.shape, pin_memory=True))
    with pytest.raises(ValueError, match="host_out"):
        solve_radiosity_batched(FF, E, 0.12, host_out=torch.empty(E.shape))
    with pytest.raises(ValueError, match="shape"):
        solve_radiosity(FF, Ep, 0.12, method="batched-bf16", out=torch.empty(3, 3))
    with pytest.raises(ValueError, match="batched methods only"):
        solve_radiosity(FF, E[:, 0].cpu().numpy(), 0.12, out=np.empty(sm.num_faces))


@pytest.fixture(scope="module")
def terrain_op():
    sm = _terrain_case(64)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    return sm, FF


@pytest.mark.parametrize("K", [256, 200, 1024])
def test_tensor_core_product_matches_mma(terrain_op, K):
    """The tcgen05 kernels (both phases) against the mma.sync kernels on the
    same BF16 operands (FP32 accumulation in both: only the summation order
    differs, and with it a rare last-bit rounding of the BF16 copy of Z), and
    both against the FP64 product."""
    sm, FF = terrain_op
    N = sm.num_faces
    g = torch.Generator(device="cuda").manual_seed(K)
    Xp = torch.rand((N, K), device="cuda", generator=g)
    Xb = Xp.to(torch.bfloat16).contiguous()
    add = torch.rand((N, K), device="cuda", generator=g)
    zr = max(FF._num_zrows, 1)
    outs = {}
    for eng in ("mma", "tc"):
        Z = torch.empty((zr, K), dtype=torch.float32, device="cuda")
        Zb = torch.empty((zr, K), dtype=torch.bfloat16, device="cuda")
        Y = torch.full((N, K), float("nan"), device="cuda")
        FF.bf16_product(Xb, Z, Zb, Y, add=add, alpha=0.5, engine=eng)
        outs[eng] = Y
    FF.check_device_flags()
    assert torch.isfinite(outs["tc"]).all()
    ref = (outs["mma"] - add).abs().max().item()
    d = (outs["tc"] - outs["mma"]).abs().max().item()
    assert d <= 2e-3 * ref, (d, ref)
    # against FP64 (BF16 rounding of operator and sources)
    Y64 = FF.matmat_permuted(Xp[:, :4].double().contiguous(), "fp64")
    yt = (outs["tc"][:, :4].double() - add[:, :4].double()) / 0.5
    assert (yt - Y64).abs().max().item() <= 2e-2 * Y64.abs().max().item()


@pytest.mark.parametrize("K", [64, 264])
def test_split_bf16_product_accuracy(terrain_op, K):
    """Split-BF16 tensor-core product of the FP32 operator against the same
    operator applied in FP64 arithmetic.  A two-part BF16 split carries ~17
    significant bits, so the product behaves like FP32 arithmetic with 7
    fewer bits (the low-rank factors amplify rounding as they do in FP32):
    within 2e-5 of max |F x| (the FP32 CUDA-core product: 5e-6).  In the
    refinement residual this is scaled by rho."""
    sm, FF = terrain_op
    N = sm.num_faces
    g = torch.Generator(device="cuda").manual_seed(K + 1)
    X = torch.rand((N, K), device="cuda", generator=g)
    Y = torch.full((N, K), float("nan"), device="cuda")
    FF.split_product(X, Y)
    FF.check_device_flags()
    Y32 = FF.matmat_permuted(X, "fp32")
    for c in (0, K // 2, K - 1):
        y64 = FF.matvec_permuted(X[:, c].double().contiguous(), "fp32-fp64")
        ref = y64.abs().max().item()
        e_split = (Y[:, c].double() - y64).abs().max().item() / ref
        e_fp32 = (Y32[:, c].double() - y64).abs().max().item() / ref
        assert e_split <= 2e-5, (c, e_split, e_fp32)
        assert e_fp32 <= 5e-6, (c, e_split, e_fp32)
    # with add / alpha
    add = torch.rand((N, K), device="cuda", generator=g)
    Y2 = torch.empty_like(Y)
    FF.split_product(X, Y2, add=add, alpha=-0.25)
    assert torch.allclose(Y2, add - 0.25 * Y, rtol=0, atol=1e-5 * Y.abs().max().item())


@pytest.mark.parametrize("K", [200, 512])
def test_tma_gather_phase_b_matches_cp_async(terrain_op, K):
    """The TMA variant of phase B (sources stacked as [Z; X], rows gathered
    by tile::gather4 in a warp-specialised kernel) against the cp.async
    kernel: the same MMA order, identical plain results; the split products
    drain their accumulators after different windows (64 rows in the TMA
    variant, 256 in the cp.async kernel), so they agree to FP32 rounding."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N = sm.num_faces
    nz = FF._num_zrows
    g = torch.Generator(device="cuda").manual_seed(K + 7)
    X = torch.rand((N, K), device="cuda", generator=g)
    add = torch.rand((N, K), device="cuda", generator=g)
    tc = FF.tc_operands(split=True)
    st = _lib.stream_handle()
    fl = _lib.ptr(FF.device_flags())
    sh = torch.empty((nz + N, K), dtype=torch.bfloat16, device="cuda")
    sl = torch.empty_like(sh)
    zf = torch.empty((max(nz, 1), K), device="cuda")
    _lib.call("fgb_split_bf16", _lib.ptr(X), _lib.ptr(sh[nz:]), _lib.ptr(sl[nz:]), N * K, st)
    _lib.call("fgb_tc_phase_a", C.byref(FF._desc_tc_items), _lib.ptr(tc["vt_hi"]), _lib.ptr(tc["vt_lo"]),
              _lib.ptr(sh[nz:]), _lib.ptr(sl[nz:]), _lib.ptr(zf), K, int(FF._needs_zero_z), fl, st)
    _lib.call("fgb_split_bf16", _lib.ptr(zf), _lib.ptr(sh[:nz]), _lib.ptr(sl[:nz]), nz * K, st)
    t64 = FF.tc_operands64(split=True)
    for split in (False, True):
        wl = _lib.ptr(t64["w_lo"]) if split else None
        Y_cp = torch.full((N, K), float("nan"), device="cuda")
        Y_tma = torch.full((N, K), float("nan"), device="cuda")
        _lib.call("fgb_tc_phase_b", C.byref(FF._desc), _lib.ptr(t64["w_hi"]), wl,
                  _lib.ptr(sh[nz:]), _lib.ptr(sl[nz:]) if split else None, _lib.ptr(sh[:nz]),
                  _lib.ptr(sl[:nz]) if split else None, _lib.ptr(Y_cp), K, _lib.ptr(add), -0.25,
                  fl, st)
        _lib.call("fgb_tc_phase_b_tma", C.byref(FF._desc), _lib.ptr(t64["w_hi"]), wl,
                  _lib.ptr(sh), _lib.ptr(sl) if split else None, _lib.ptr(Y_tma), K,
                  _lib.ptr(add), -0.25, fl, st)
        FF.check_device_flags()
        assert torch.isfinite(Y_tma).all()
        if split:
            # one or two roundings of Y itself (|Y| ~ 1, |alpha F x| ~ 0.1)
            ref = Y_cp.abs().max().item()
            assert (Y_tma - Y_cp).abs().max().item() <= 1e-6 * ref
        else:
            assert torch.equal(Y_tma, Y_cp)


@pytest.mark.parametrize("slice_rows", [128, 64])
def test_phase_a_bf16_output_matches_fp32(terrain_op, slice_rows):
    """Phase A with whole-group work items writing Z as BF16 hi / lo parts
    (work slices of 128 rows, or of 64 rows with two CTAs per SM) against
    phase A with column-split items accumulating FP32 Z."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N, K = sm.num_faces, 136
    nz = FF._num_zrows
    g = torch.Generator(device="cuda").manual_seed(11)
    X = torch.rand((N, K), device="cuda", generator=g)
    tc = FF.tc_operands(split=True)
    st = _lib.stream_handle()
    fl = _lib.ptr(FF.device_flags())
    xh = torch.empty((N, K), dtype=torch.bfloat16, device="cuda")
    xl = torch.empty_like(xh)
    _lib.call("fgb_split_bf16", _lib.ptr(X), _lib.ptr(xh), _lib.ptr(xl), N * K, st)
    z32 = torch.empty((nz, K), device="cuda")
    _lib.call("fgb_tc_phase_a", C.byref(FF._desc_tc_items), _lib.ptr(tc["vt_hi"]), _lib.ptr(tc["vt_lo"]),
              _lib.ptr(xh), _lib.ptr(xl), _lib.ptr(z32), K, int(FF._needs_zero_z), fl, st)
    zh = torch.full((nz, K), float("nan"), dtype=torch.bfloat16, device="cuda")
    zl = torch.full_like(zh, float("nan"))
    desc = FF._desc_tc if slice_rows == 128 else FF._desc_tc64
    assert desc.slice_rows == slice_rows
    _lib.call("fgb_tc_phase_a_bf16", C.byref(desc), _lib.ptr(tc["vt_hi"]),
              _lib.ptr(tc["vt_lo"]), _lib.ptr(xh), _lib.ptr(xl), _lib.ptr(zh), _lib.ptr(zl), K,
              fl, st)
    FF.check_device_flags()
    z = zh.float() + zl.float()
    assert torch.isfinite(z).all()
    assert (z - z32).abs().max().item() <= 1e-5 * z32.abs().max().item()
    if slice_rows == 64:
        # the plain product takes 128-row slices only
        with pytest.raises(ValueError, match="128-row work slices"):
            _lib.call("fgb_tc_phase_a_bf16", C.byref(desc), _lib.ptr(tc["vt_hi"]), None,
                      _lib.ptr(xh), None, _lib.ptr(zh), None, K, fl, st)


@pytest.mark.parametrize("K", [3, 5, 132])
def test_fp32_multi_rhs_product_any_width(terrain_op, K):
    """The FP32 CUDA-core K-column product (16-byte gathers when K % 4 == 0,
    4-byte gathers otherwise) against the FP64 product."""
    sm, FF = terrain_op
    g = torch.Generator(device="cuda").manual_seed(K + 3)
    X = torch.rand((sm.num_faces, K), device="cuda", generator=g, dtype=torch.float64)
    Y32 = FF.matmat_permuted(X.float().contiguous(), "fp32")
    Y64 = FF.matmat_permuted(X, "fp64")
    assert (Y32.double() - Y64).abs().max().item() <= 5e-6 * Y64.abs().max().item()


@pytest.mark.parametrize("K", [256, 520])
def test_phase_b_128_row_tiles_match_64(terrain_op, K):
    """The plain BF16 phase B on the re-tiled 128-row panel (rows of tiles
    2t and 2t + 1 that gather the same source merged) against the 64-row
    panel: same products, summed in another order."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N = sm.num_faces
    nz = FF._num_zrows
    tc = FF.tc_operands(split=True)
    g = torch.Generator(device="cuda").manual_seed(K + 5)
    S = torch.rand((nz + N, K), device="cuda", generator=g).to(torch.bfloat16)
    add = torch.rand((N, K), device="cuda", generator=g)
    fl = _lib.ptr(FF.device_flags())
    st = _lib.stream_handle()
    Y64 = torch.full((N, K), float("nan"), device="cuda")
    Y128 = torch.full((N, K), float("nan"), device="cuda")
    _lib.call("fgb_tc_phase_b", C.byref(FF._desc), _lib.ptr(FF.tc_operands64()["w_hi"]), None,
              _lib.ptr(S[nz:]), None, _lib.ptr(S[:nz]), None, _lib.ptr(Y64), K, _lib.ptr(add),
              0.5, fl, st)
    _lib.call("fgb_tc_phase_b", C.byref(FF._desc128), _lib.ptr(tc["w128"]), None,
              _lib.ptr(S[nz:]), None, _lib.ptr(S[:nz]), None, _lib.ptr(Y128), K, _lib.ptr(add),
              0.5, fl, st)
    FF.check_device_flags()
    assert torch.isfinite(Y128).all()
    ref = (Y64 - add).abs().max().item()
    assert (Y128 - Y64).abs().max().item() <= 1e-5 * ref
    assert FF.stats["panel_rows_128"] > 0


@pytest.mark.parametrize("K", [256, 520])
def test_phase_b_256_row_tiles_match_64(terrain_op, K):
    """The plain BF16 phase B on the 256-row panel (rows of the four 64-row
    tiles 4t .. 4t + 3 that gather the same source merged; MMA N = 256)
    against the 64-row panel: same products, summed in another order; the
    256-row layout has at most as many rows as the 128-row one."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N = sm.num_faces
    nz = FF._num_zrows
    tc = FF.tc_operands256()
    g = torch.Generator(device="cuda").manual_seed(K + 7)
    S = torch.rand((nz + N, K), device="cuda", generator=g).to(torch.bfloat16)
    add = torch.rand((N, K), device="cuda", generator=g)
    fl = _lib.ptr(FF.device_flags())
    st = _lib.stream_handle()
    Y64 = torch.full((N, K), float("nan"), device="cuda")
    Y256 = torch.full((N, K), float("nan"), device="cuda")
    _lib.call("fgb_tc_phase_b", C.byref(FF._desc), _lib.ptr(FF.tc_operands64()["w_hi"]), None,
              _lib.ptr(S[nz:]), None, _lib.ptr(S[:nz]), None, _lib.ptr(Y64), K, _lib.ptr(add),
              0.5, fl, st)
    assert FF._desc256.tile_rows == 256
    _lib.call("fgb_tc_phase_b", C.byref(FF._desc256), _lib.ptr(tc["w256"]), None,
              _lib.ptr(S[nz:]), None, _lib.ptr(S[:nz]), None, _lib.ptr(Y256), K, _lib.ptr(add),
              0.5, fl, st)
    FF.check_device_flags()
    assert torch.isfinite(Y256).all()
    ref = (Y64 - add).abs().max().item()
    assert (Y256 - Y64).abs().max().item() <= 1e-5 * ref
    assert 0 < FF.stats["panel_rows_256"] <= FF.stats["panel_rows_128"] + 64 * FF._desc256.num_tiles
    # the product through the plan that uses it (phase A writes Z into
    # S[:nz], then the 256-row phase B runs on S)
    plan = FF.product_plan()
    old = dict(plan)
    try:
        plan["plain"] = "b256"
        Y = torch.empty_like(Y64)
        FF.bf16_product(S[nz:], None, S[:nz], Y, add=add, alpha=0.5)
        _lib.call("fgb_tc_phase_b", C.byref(FF._desc256), _lib.ptr(tc["w256"]), None,
                  _lib.ptr(S[nz:]), None, _lib.ptr(S[:nz]), None, _lib.ptr(Y256), K,
                  _lib.ptr(add), 0.5, fl, st)
        FF.check_device_flags()
        assert torch.equal(Y, Y256)
    finally:
        plan.update(old)


@pytest.mark.parametrize("split", [False, True])
def test_phase_b_separate_sources_match_stacked(terrain_op, split):
    """fgb_tc_phase_b with Z and X in separate buffers (a row select per
    gathered row) against the same call on one stacked [Z; X] tensor (one
    base pointer): identical results."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N, K = sm.num_faces, 264
    nz = FF._num_zrows
    tc = FF.tc_operands(split=True)
    g = torch.Generator(device="cuda").manual_seed(31 + split)
    Sh = torch.rand((nz + N, K), device="cuda", generator=g).to(torch.bfloat16)
    Sl = (torch.rand((nz + N, K), device="cuda", generator=g) * 1e-3).to(torch.bfloat16)
    Zh, Xh = Sh[:nz].clone(), Sh[nz:].clone()
    Zl, Xl = Sl[:nz].clone(), Sl[nz:].clone()
    add = torch.rand((N, K), device="cuda", generator=g)
    fl = _lib.ptr(FF.device_flags())
    st = _lib.stream_handle()
    desc = FF._desc if split else FF._desc128
    w_hi = tc["w_hi"] if split else tc["w128"]
    w_lo = _lib.ptr(tc["w_lo"]) if split else None
    Y1 = torch.full((N, K), float("nan"), device="cuda")
    Y2 = torch.full((N, K), float("nan"), device="cuda")
    _lib.call("fgb_tc_phase_b", C.byref(desc), _lib.ptr(w_hi), w_lo,
              _lib.ptr(Sh[nz:]), _lib.ptr(Sl[nz:]) if split else None,
              _lib.ptr(Sh[:nz]), _lib.ptr(Sl[:nz]) if split else None,
              _lib.ptr(Y1), K, _lib.ptr(add), 0.5, fl, st)
    _lib.call("fgb_tc_phase_b", C.byref(desc), _lib.ptr(w_hi), w_lo,
              _lib.ptr(Xh), _lib.ptr(Xl) if split else None,
              _lib.ptr(Zh), _lib.ptr(Zl) if split else None,
              _lib.ptr(Y2), K, _lib.ptr(add), 0.5, fl, st)
    FF.check_device_flags()
    assert torch.isfinite(Y1).all()
    assert torch.equal(Y1, Y2)


def test_phase_a_slice_item_table_matches_search(terrain_op):
    """Tensor-core phase A with the per-slice item table (a_witem) against
    the same descriptor without it (item found by binary search over
    a_woff): identical BF16 Z."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    from fluxpy_gb300.compressed_form_factors import fgb_op_desc
    sm, FF = terrain_op
    N, K = sm.num_faces, 128
    nz = FF._num_zrows
    tc = FF.tc_operands(split=True)
    g = torch.Generator(device="cuda").manual_seed(41)
    X = torch.rand((N, K), device="cuda", generator=g).to(torch.bfloat16)
    fl = _lib.ptr(FF.device_flags())
    st = _lib.stream_handle()
    bare = fgb_op_desc.from_buffer_copy(FF._desc_tc)
    bare.a_witem = None
    assert FF._desc_tc.a_witem
    Z1 = torch.full((nz, K), float("nan"), dtype=torch.bfloat16, device="cuda")
    Z2 = torch.full_like(Z1, float("nan"))
    for desc, Z in ((FF._desc_tc, Z1), (bare, Z2)):
        _lib.call("fgb_tc_phase_a_bf16", C.byref(desc), _lib.ptr(tc["vt_hi"]), None,
                  _lib.ptr(X), None, _lib.ptr(Z), None, K, fl, st)
    FF.check_device_flags()
    assert torch.isfinite(Z1.float()).all()
    assert torch.equal(Z1, Z2)


def test_split_phase_b_128_row_tiles_match_64(terrain_op):
    """The split-BF16 phase B on the re-tiled 128-row panel (hi and lo
    parts, 16 warps per CTA) against the 64-row panel: the same products
    summed in another order, within the split product's rounding."""
    import ctypes as C
    from fluxpy_gb300 import _lib
    sm, FF = terrain_op
    N, K = sm.num_faces, 256
    nz = FF._num_zrows
    t64 = FF.tc_operands64(split=True)
    w128, w128_lo = FF.tc_split128()
    g = torch.Generator(device="cuda").manual_seed(53)
    X = torch.rand((nz + N, K), device="cuda", generator=g)
    Sh = torch.empty((nz + N, K), dtype=torch.bfloat16, device="cuda")
    Sl = torch.empty_like(Sh)
    st = _lib.stream_handle()
    _lib.call("fgb_split_bf16", _lib.ptr(X), _lib.ptr(Sh), _lib.ptr(Sl), (nz + N) * K, st)
    fl = _lib.ptr(FF.device_flags())
    Y64 = torch.full((N, K), float("nan"), device="cuda")
    Y128 = torch.full((N, K), float("nan"), device="cuda")
    for desc, wh, wl, Y in ((FF._desc, t64["w_hi"], t64["w_lo"], Y64),
                            (FF._desc128, w128, w128_lo, Y128)):
        _lib.call("fgb_tc_phase_b", C.byref(desc), _lib.ptr(wh), _lib.ptr(wl),
                  _lib.ptr(Sh[nz:]), _lib.ptr(Sl[nz:]), _lib.ptr(Sh[:nz]), _lib.ptr(Sl[:nz]),
                  _lib.ptr(Y), K, None, 1.0, fl, st)
    FF.check_device_flags()
    assert torch.isfinite(Y128).all()
    ref = Y64.abs().max().item()
    assert (Y128 - Y64).abs().max().item() <= 2e-6 * ref
