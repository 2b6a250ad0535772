"""GPU: the exact triangle-triangle view factor (fgb_ff_triangles_f64,
fluxpy_gb300.view_factor) against the reference's own C
(src/flux/view_factor/view_factor_narayanaswamy.c, its outputs in
tests/golden/viewfactor.npz) and against brute-force quadrature of the
defining double integral (oracle/viewfactor.py), and its use as the
near-field correction of get_form_factor_matrix."""
import numpy as np
import pytest

from fluxpy_gb300 import shape as gshape, terrain
from fluxpy_gb300.form_factors import get_form_factor_matrix
from fluxpy_gb300.view_factor import ff_narayanaswamy, ff_triangles
from oracle import viewfactor as ovf
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN / "viewfactor.npz")


def test_matches_reference_c(golden):
    F = ff_triangles(golden["T1"], golden["T2"])
    ref = golden["F"]
    rel = np.abs(F - ref) / np.abs(ref)
    # the nine edge-pair terms of the closed form are much larger than their
    # sum (most for parallel edges), so two FP64 evaluations in different
    # operation orders agree to ~1e-8 relative, not to the last bit; for two
    # nearly coplanar triangles that share an edge (normals 0.14 degrees
    # apart, F = 4.3e-7) the sum cancels to 7 digits below its terms and the
    # two evaluations differ by 4e-11 absolute (1e-4 relative), below what
    # brute-force quadrature of that singular pair can resolve
    bound = np.maximum(1e-7 * np.abs(ref), 1e-10)
    for kind in np.unique(golden["kind"]):
        sel = golden["kind"] == kind
        assert np.all(np.abs(F - ref)[sel] <= bound[sel]), (kind, rel[sel].max())
    assert np.median(rel) < 1e-11


def test_drop_in_single_pair(golden):
    for q in (0, 151, 399):
        assert abs(ff_narayanaswamy(golden["T1"][q], golden["T2"][q]) - golden["F"][q]) <= \
            1e-9 * golden["F"][q]
    with pytest.raises(ValueError):
        ff_narayanaswamy(np.zeros((4, 3)), np.zeros((3, 3)))


def test_separated_pairs_match_quadrature(golden):
    # the defining integral by brute force: O(h^2), two levels extrapolated
    sel = np.flatnonzero(golden["kind"] == "separated")[:6]
    F = ff_triangles(golden["T1"][sel], golden["T2"][sel])
    for q, f in zip(sel, F):
        a, b = golden["T1"][q], golden["T2"][q]
        q5, q6 = ovf.ff_quadrature(a, b, 5), ovf.ff_quadrature(a, b, 6)
        rich = q6 + (q6 - q5) / 3
        assert abs(f - rich) <= 5e-5 * f, (q, f, rich)


def test_adjacent_correction_of_the_form_factor_matrix():
    V, Fc = terrain.spherical_crater(n_points=300, seed=0, boundary_grid=12)
    sm = gshape.EmbreeTrimeshShapeModel(V, Fc)
    A = get_form_factor_matrix(sm).tocoo()
    B = get_form_factor_matrix(sm, exact_adjacent=True).tocoo()
    assert np.array_equal(A.row, B.row) and np.array_equal(A.col, B.col)
    shared = np.array([np.intersect1d(Fc[i], Fc[j]).size > 0 for i, j in zip(A.row, A.col)])
    assert shared.any()
    # untouched away from adjacent facets; adjacent entries are the kernel's
    assert np.array_equal(A.data[~shared], B.data[~shared])
    want = ff_triangles(V[Fc[A.row[shared]]], V[Fc[A.col[shared]]])
    assert np.allclose(B.data[shared], want, rtol=1e-13, atol=0)
