"""GPU: the product autotuner (CompressedFormFactorMatrix.autotune_products)
times every kernel layout of the BF16 and split-BF16 products, keeps the
fastest, and every layout computes the same product."""
import numpy as np
import pytest
import torch

from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                  FormFactorOctreeBlock)
from fluxpy_gb300.solve import solve_radiosity_batched

pytestmark = pytest.mark.gpu


def test_autotuned_plans_agree_and_solve():
    V, F = terrain.fbm_terrain(n=48, seed=5, n_craters=4)
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=4096, dtype=np.float32,
                                    RootBlock=FormFactorOctreeBlock)
    K = 64
    table = FF.autotune_products(K, reps=2)
    for kind, plans in (("plain", FF.PLAIN_PLANS), ("split", FF.SPLIT_PLANS)):
        assert set(table[kind]) == set(plans)
        timed = {p: t for p, t in table[kind].items() if t is not None}
        # the fastest layout (ties: any of them)
        assert timed[table["chosen"][kind]] == min(timed.values())
    assert FF.product_plan() == table["chosen"]
    # every layout: the same product as the FP64 one, to BF16 / split accuracy
    rng = np.random.default_rng(0)
    X = torch.as_tensor(rng.uniform(0, 1, (sm.num_faces, K)), dtype=torch.float32,
                        device="cuda")
    Xp = FF.permute(X).contiguous()
    ref = FF.matmat_permuted(Xp[:, :4].double().contiguous(), "fp64")
    scale = ref.abs().max().item()
    chosen = dict(FF.product_plan())
    Y = torch.empty_like(Xp)
    Sb, Zb, Xb = FF.stacked_sources(K, Xp.device)
    Xb.copy_(Xp)
    for p in FF.PLAIN_PLANS:
        FF.product_plan()["plain"] = p
        FF.bf16_product(Xb, None, Zb, Y)
        assert (Y[:, :4].double() - ref).abs().max().item() / scale < 2e-2, p
    for p in FF.SPLIT_PLANS:
        FF.product_plan()["split"] = p
        FF.split_product(Xp, Y)
        assert (Y[:, :4].double() - ref).abs().max().item() / scale < 2e-5, p
    FF.check_device_flags()
    FF.product_plan().update(chosen)
    # the solver with the chosen layouts
    dirs = terrain.random_sun_directions(K, seed=2)
    E = sm.get_direct_irradiance_batch(1365.0, dirs, out_dtype=torch.float32)
    st = {}
    B = solve_radiosity_batched(FF, E, 0.12, rtol=1e-5, stats=st)
    Bp = FF.permute(B.double())
    FBp = FF.matmat_permuted((0.12 * Bp[:, :4]).contiguous(), "fp64")
    Ep = FF.permute(E.double())[:, :4]
    R = Ep - (Bp[:, :4] - FBp)
    assert (R.abs().amax(0) / Ep.abs().amax(0).clamp_min(1e-30)).max().item() <= 1e-5, st
