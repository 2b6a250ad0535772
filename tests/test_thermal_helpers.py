"""CPU: setgrid, flux_noatm and analytT_ (thermal.pyx:301-396) equal the
reference's own values on fixed inputs (tests/golden/thermal_helpers.npz,
made by tests/golden/make_golden.py from the reference's source)."""
import numpy as np

from fluxpy_gb300.thermal import analytT_, flux_noatm, setgrid
from tests.conftest import GOLDEN
from tests.golden.make_golden import thermal_helper_cases


def test_thermal_helpers_match_reference_values():
    g = np.load(GOLDEN / "thermal_helpers.npz")
    grids, flux, analyt = thermal_helper_cases()
    z = np.split(g["setgrid"], np.cumsum(g["setgrid_len"])[:-1])
    for args, ref in zip(grids, z):
        got = setgrid(*args)
        assert got.shape == ref.shape and np.array_equal(got, ref), args
    F = np.array([flux_noatm(*row) for row in flux])
    assert np.array_equal(F, g["flux_noatm"])
    assert (F > 0).any() and (F == 0).any()          # lit and unlit cases both present
    assert np.array_equal(analytT_(**analyt), g["analytT"])
