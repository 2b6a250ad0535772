"""The PCC golden scenario of the reference's tests/test_thermal.py:33-77,
with the constructor call adapted to the current PccThermalModel1D signature
(thermal.pyx:89-98): the test there still passes the removed keywords
``nfaces=``, ``emissivity=`` and ``Qprev=``.  With z = [0, setgrid(60, 1.05,
2.5)], ti = 120, rhoc = 9.6e5, emiss = 1, Fgeotherm = 0.2 and Q0 = Qn the
scenario reproduces the reference's golden files."""
from __future__ import annotations

import numpy as np

NZ = 60
ZFAC = 1.05
ZMAX = 2.5
STEPSPERSOL = 120
PERIOD = 88775.244 * 670
ALBEDO = 0.2
RAU = 1.52
LATITUDE = np.deg2rad(5.0)
DT = 495661.77900000004
NSTEPS = 50000


def grid(setgrid):
    return np.concatenate([[0.0], setgrid(nz=NZ, zfac=ZFAC, zmax=ZMAX)])


def fluxes(flux_noatm):
    """Qn and the Qnp1 sequence of the scenario (test_thermal.py:41-63)."""
    Qn = (1 - ALBEDO) * flux_noatm(RAU, 0.0, LATITUDE, 0.0, 0.0, 0.0)
    q = np.empty(NSTEPS + 1)
    for i in range(NSTEPS + 1):
        time = (i + 1) * DT
        HA = 2 * np.pi * (time / PERIOD % 1.0)
        q[i] = (1 - ALBEDO) * flux_noatm(RAU, 0.0, LATITUDE, HA, 0.0, 0.0)
    return Qn, q


def run(step, get_T, Qnp1_seq):
    """Drive ``step(i, dt)`` (advancing with Qnp1_seq[i]) and collect the
    outputs the golden files hold (test_thermal.py:56-77)."""
    Tsurface_output, Tprofile_output = [], []
    for i in range(NSTEPS + 1):
        time = (i + 1) * DT
        step(i, DT)
        if i % 3 == 0:
            T = get_T()
            Tsurface_output.append([time / PERIOD, T[0], T[NZ]])
        if i > NSTEPS - STEPSPERSOL and i % 10 == 0:
            Tprofile_output.append(np.array(get_T()))
    return np.vstack(Tprofile_output)[-1], np.vstack(Tsurface_output)


def check_against_golden(Tprofile_out, Tsurface_out, golden):
    Tprofile = golden["Tprofile"][-1]
    Tsurface = golden["Tsurface"]
    # the reference's own criteria (test_thermal.py:98-101)
    assert abs(np.sum(np.round(Tprofile_out, 3) - np.round(Tprofile, 3))) < 1e-3
    assert abs(np.sum(np.round(Tsurface_out, 3) - np.round(Tsurface, 3))) < 1e-3
    # and elementwise: the golden files hold 3 decimals
    assert np.max(np.abs(Tprofile_out - Tprofile)) <= 5.0e-4 + 1e-9
    assert np.max(np.abs(Tsurface_out[:, 1:] - Tsurface[:, 1:])) <= 5.0e-4 + 1e-9
    assert np.max(np.abs(Tsurface_out[:, 0] - Tsurface[:, 0])) <= 5.0e-7 + 1e-12
