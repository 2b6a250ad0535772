"""CPU: the reference's exact triangle view factors (tests/golden/
viewfactor.npz, made from src/flux/view_factor/view_factor_narayanaswamy.c)
against brute-force quadrature of the defining double integral
(oracle/viewfactor.py), and against the reference's C itself where
oracle/_ref holds it."""
import numpy as np
import pytest

from oracle import viewfactor as ovf
from tests.conftest import GOLDEN


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN / "viewfactor.npz")


def test_golden_separated_pairs_match_quadrature(golden):
    sel = np.flatnonzero(golden["kind"] == "separated")[::30]
    for q in sel:
        a, b = golden["T1"][q], golden["T2"][q]
        q4, q5 = ovf.ff_quadrature(a, b, 4), ovf.ff_quadrature(a, b, 5)
        rich = q5 + (q5 - q4) / 3
        assert abs(golden["F"][q] - rich) <= 1e-4 * golden["F"][q]


def test_golden_parallel_pairs_match_quadrature(golden):
    sel = np.flatnonzero(golden["kind"] == "parallel")[::10]
    for q in sel:
        a, b = golden["T1"][q], golden["T2"][q]
        q4, q5 = ovf.ff_quadrature(a, b, 4), ovf.ff_quadrature(a, b, 5)
        rich = q5 + (q5 - q4) / 3
        assert abs(golden["F"][q] - rich) <= 1e-4 * golden["F"][q]


def test_golden_is_the_reference_c(golden):
    if ovf.ff_ref(golden["T1"][0], golden["T2"][0]) is None:
        pytest.skip("oracle/_ref not built (no reference tree here)")
    for q in range(0, golden["F"].size, 7):
        assert ovf.ff_ref(golden["T1"][q], golden["T2"][q]) == golden["F"][q]
