"""GPU: uneven batches of independent meshes (fluxpy_gb300/batch.py): the
merged block-diagonal operator against each mesh's own product, and the
batched FP32 thermal model (eager and CUDA-graph replay) against one
ThermalModel per mesh (src/flux/model.py:108-234), which is itself checked
against the reference's iteration in test_gpu_model.py."""
import numpy as np
import pytest
import torch

from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.batch import BlockDiagonalOperator, MultiMeshThermalModel
from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                  FormFactorOctreeBlock)
from fluxpy_gb300.model import ThermalModel
from fluxpy_gb300.thermal import setgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def meshes():
    out = []
    for n_points, grid, seed in ((300, 10, 11), (900, 16, 12), (1800, 20, 13)):
        V, F = terrain.spherical_crater(n_points=n_points, seed=seed, boundary_grid=grid)
        sm = gshape.EmbreeTrimeshShapeModel(V, F)
        FF = CompressedFormFactorMatrix(sm, tol=1e-5, min_size=1024, dtype=np.float32,
                                        RootBlock=FormFactorOctreeBlock)
        out.append((sm, FF))
    assert any(FF.stats["lowrank_blocks"] > 0 for _, FF in out)
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_block_diagonal_product_matches_each_mesh(meshes, precision):
    ops = [FF for _, FF in meshes]
    bd = BlockDiagonalOperator(ops, precision)
    assert bd.num_faces == sum(FF.num_faces for FF in ops)
    assert bd.num_rows % 64 == 0
    rng = np.random.default_rng(0)
    dt = torch.float64 if precision == "fp64" else torch.float32
    x = torch.as_tensor(rng.uniform(0, 1, bd.num_faces), dtype=dt, device="cuda")
    y = bd @ x
    parts, o = [], 0
    for FF in ops:
        xi = x[o:o + FF.num_faces]
        parts.append(FF.unpermute(FF.matvec_permuted(FF.permute(xi), precision)))
        o += FF.num_faces
    ref = torch.cat(parts)
    if not bd._needs_zero_z:
        # same kernels, same tiles, same order of sums
        assert torch.equal(y, ref)
    else:
        assert torch.allclose(y, ref, rtol=1e-6, atol=0)
    # padding rows of the merged cluster order stay zero
    yc = bd.matvec_cluster(bd.to_cluster(x))
    pad = torch.ones(bd.num_rows, dtype=torch.bool, device="cuda")
    pad[bd.cluster_row] = False
    assert torch.count_nonzero(yc[pad]).item() == 0


def _sun(nt):
    elev = np.deg2rad(np.linspace(8.0, 40.0, nt))
    az = np.deg2rad(np.linspace(0.0, 75.0, nt))
    return np.column_stack([np.cos(elev) * np.cos(az), np.cos(elev) * np.sin(az), np.sin(elev)])


def test_multi_mesh_model_matches_thermal_model_per_mesh(meshes):
    nt = 10
    t = np.linspace(0.0, 9 * 3600.0, nt)
    D = _sun(nt)
    F0 = np.full(nt, 1365.0)
    rho, emiss, Fg, T0 = 0.12, 0.95, 0.005, 210.0
    z = np.concatenate([[0.0], setgrid(20, 1.08, 0.5)])
    ti = np.linspace(55.0, 400.0, z.size)
    rhoc = np.full(z.size, 960000.0)
    ops = [FF for _, FF in meshes]
    kw = dict(rho=rho, z=z, ti=ti, rhoc=rhoc, emiss=emiss, Fgeotherm=Fg, T0=T0)
    mg = MultiMeshThermalModel(ops, t, D, F0, use_graph=True, **kw)
    me = MultiMeshThermalModel(ops, t, D, F0, use_graph=False, **kw)
    Tg = mg.run()
    Te = me.run()
    mg.check_errors()
    assert mg._graph is not None
    # the graph replays exactly the eager launches
    assert torch.equal(Tg, Te)
    assert torch.equal(mg.T, me.T)
    # against one FP64 ThermalModel per mesh
    o = 0
    for sm, FF in meshes:
        m = ThermalModel(FF, t, D, F0, rho, z=z, T0=T0, ti=ti, rhoc=rhoc, emiss=emiss,
                         Fgeotherm=Fg, shape_model=sm)
        T = None
        for T in m:
            pass
        got = mg.T[o:o + FF.num_faces].double().cpu().numpy()
        err = np.max(np.abs(got - T))
        assert err < 5e-3, err
        o += FF.num_faces
    # stepping in pieces gives the same result as one run
    mp = MultiMeshThermalModel(ops, t, D, F0, use_graph=True, **kw)
    mp.run(3)
    mp.run(2)
    mp.run()
    assert torch.equal(mp.T, mg.T)
