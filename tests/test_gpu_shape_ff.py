"""GPU parity of the shape model, LBVH ray queries and the form-factor pair
kernel against the oracle (bit-exact) and the reference's invariants."""
import numpy as np
import pytest
import scipy.sparse

from oracle import vis
from tests.conftest import GOLDEN
from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.form_factors import get_form_factor_matrix, get_form_factor_matrix_device

pytestmark = pytest.mark.gpu

SEMS = [(gshape.EmbreeTrimeshShapeModel, vis.EMBREE), (gshape.CgalTrimeshShapeModel, vis.CGAL)]


@pytest.fixture(scope="module")
def spheres():
    return np.load(GOLDEN / "spheres.npz")


@pytest.fixture(scope="module")
def crater():
    return terrain.spherical_crater()


@pytest.fixture(scope="module")
def small_terrain():
    return terrain.fbm_terrain(n=48, seed=11, n_craters=4)


def test_geometry_bitwise_vs_numpy(crater, small_terrain):
    for V, F in (crater, small_terrain):
        sm = gshape.EmbreeTrimeshShapeModel(V, F)
        P, N, A = vis.geometry(V, F)
        assert np.array_equal(sm.P, P)
        assert np.array_equal(sm.N, N)
        assert np.array_equal(sm.A, A)
    V32 = crater[0].astype(np.float32)
    sm = gshape.EmbreeTrimeshShapeModel(V32, crater[1])
    P, N, A = vis.geometry(V32, crater[1])
    assert sm.P.dtype == np.float32
    assert np.array_equal(sm.P, P) and np.array_equal(sm.N, N) and np.array_equal(sm.A, A)


@pytest.mark.parametrize("cls,sem", SEMS)
@pytest.mark.parametrize("name", ["icosa_sphere", "icosa_sphere_5"])
def test_reference_sphere_visibility(spheres, cls, sem, name):
    # tests/test_shape.py:16-60
    V, F = spheres[f"{name}_V"], spheres[f"{name}_F"]
    sm = cls(V, F)
    sm.N[(sm.N * sm.P).sum(1) < 0] *= -1
    n = sm.num_faces
    gt = (np.ones((n, n)) - np.eye(n)).astype(bool)
    vis_m = sm.get_visibility_matrix(oriented=False)
    if sem == vis.EMBREE:
        gt_u = gt | np.eye(n, dtype=bool)  # Embree forces i == j visible
    else:
        gt_u = gt
    assert (vis_m == gt_u).all()
    assert (sm.get_visibility_matrix(oriented=True) == False).all()
    sm.N *= -1
    # the orientation filter (shape.py:157-161) drops i == j (P_j - P_i = 0)
    assert (sm.get_visibility_matrix(oriented=True) == gt).all()
    # get_visibility == rows of get_visibility_1_to_N (test_shape.py:86-115)
    I = np.arange(n)
    v = sm.get_visibility(I, I)
    for i in range(0, n, 37):
        assert (sm.get_visibility_1_to_N(i, I) == v[i]).all()


@pytest.mark.parametrize("cls,sem", SEMS)
def test_visibility_bitwise_vs_oracle(crater, small_terrain, cls, sem):
    for V, F in (crater, small_terrain):
        sm = cls(V, F)
        s = vis.Scene(V, F)
        rng = np.random.default_rng(0)
        n = sm.num_faces
        I = rng.choice(n, 60, replace=False)
        J = np.arange(n)
        g = sm.get_visibility(I, J)
        o = s.visibility(sm.P, I, J, sem=sem)
        assert np.array_equal(g, o), np.argwhere(g != o)[:10]
        assert 0 < g.mean() < 1


@pytest.mark.parametrize("cls,sem", SEMS)
def test_occlusion_and_irradiance_vs_oracle(crater, small_terrain, cls, sem):
    dirs = terrain.sun_directions([10.0, 3.0, 25.0], [0.0, 130.0, 260.0])
    for V, F in (crater, small_terrain):
        sm = cls(V, F)
        s = vis.Scene(V, F)
        I = np.arange(sm.num_faces)
        for d in dirs:
            assert np.array_equal(sm.is_occluded(I, d), s.occluded(sm.P, sm.N, I, d, sem=sem))
            E = sm.get_direct_irradiance(1365.0, d)
            occ = s.occluded(sm.P, sm.N, I, d, sem=sem)
            Eo = np.where(~occ, 1365.0 * np.maximum(0, sm.N @ d), 0.0)
            assert np.allclose(E, Eo, rtol=1e-13, atol=1e-9)
        Eb = sm.get_direct_irradiance_batch(1365.0, dirs, device_out=False)
        for k, d in enumerate(dirs):
            assert np.allclose(Eb[:, k], sm.get_direct_irradiance(1365.0, d), rtol=1e-13, atol=1e-9)


@pytest.mark.parametrize("cls,sem", SEMS)
def test_form_factor_matrix_bitwise_vs_oracle(crater, small_terrain, cls, sem):
    for V, F in (crater, small_terrain):
        sm = cls(V, F)
        s = vis.Scene(V, F)
        Fg = get_form_factor_matrix(sm)
        Fo = s.ff_csr(sm.P, sm.N, sm.A, sem=sem)
        assert Fg.shape == Fo.shape
        assert np.array_equal(Fg.indptr, Fo.indptr)
        assert np.array_equal(Fg.indices, Fo.indices)
        assert np.array_equal(Fg.data, Fo.data)
        # sub-blocks with arbitrary index sets: column indices are positions in J
        rng = np.random.default_rng(1)
        I = rng.choice(sm.num_faces, 50, replace=False)
        J = rng.choice(sm.num_faces, 700, replace=False)
        Fs = get_form_factor_matrix(sm, I, J)
        Fso = s.ff_csr(sm.P, sm.N, sm.A, I, J, sem=sem)
        assert np.array_equal(Fs.toarray(), Fso.toarray())


def test_form_factor_matrix_vs_reference_python(crater):
    ref = np.load(GOLDEN / "ffref.npz")
    V, F = ref["crater_V"], ref["crater_F"]
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    Fg = get_form_factor_matrix(sm)
    n = sm.num_faces
    R = scipy.sparse.csr_matrix((ref["crater_data"], ref["crater_indices"], ref["crater_indptr"]),
                                shape=(len(ref["crater_indptr"]) - 1, n))
    G = Fg[0::16]
    diff = (G != 0).astype(int) - (R != 0).astype(int)
    assert abs(diff).sum() <= 2
    assert abs(Fg.nnz - int(ref["crater_nnz"])) <= 32
    assert np.allclose(np.asarray(Fg.sum(1)).ravel(), ref["crater_rowsum"], rtol=1e-9, atol=1e-12)
    # inward sphere: all off-diagonal entries nonzero (tests/test_form_factors.py:18-38)
    sm2 = gshape.EmbreeTrimeshShapeModel(ref["sphere_V"], ref["sphere_F"])
    sm2.N[(sm2.P * sm2.N).sum(1) > 0] *= -1
    Fs = get_form_factor_matrix(sm2).toarray()
    off = ~np.eye(sm2.num_faces, dtype=bool)
    assert (Fs.diagonal() == 0).all() and (Fs[off] != 0).all()
    sm2.N *= -1
    assert get_form_factor_matrix(sm2).nnz == 0


def test_form_factor_near_edge_and_stats(small_terrain):
    V, F = small_terrain
    sm = gshape.EmbreeTrimeshShapeModel(V, F)
    t = get_form_factor_matrix_device(sm)
    assert t.kept_pairs >= t.data.numel()
    assert t.near_edge_pairs >= 0
