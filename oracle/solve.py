"""ORACLE — radiosity solves and steady-state temperatures on the CPU
(test infrastructure; also the CPU baseline of bench.py).

Restates src/flux/solve.py:4-45 (Jacobi, right/left albedo placement, default
tolerance finfo(E.dtype).resolution * max|E|, one global stopping test,
returning the iterate before the converged update) and
src/flux/model.py:8-42 (compute_steady_state_temp) with numpy/scipy
operators.  Pinned against the reference's own outputs in
tests/golden/ffref.npz (tests/test_oracle_solve.py).
"""
import numpy as np
from scipy.constants import Stefan_Boltzmann as sigSB


def solve_radiosity(FF, E, rho=1, albedo_placement="right", tol=None, max_iter=100000):
    if tol is None:
        tol = np.finfo(E.dtype).resolution * abs(E).max()
    B = E.copy()
    niter = 0
    while True:
        niter += 1
        if albedo_placement == "right":
            B1 = E + FF @ (rho * B)
        else:
            B1 = E + rho * (FF @ B)
        if abs(B1 - B).max() <= tol:
            return B, niter
        B = B1
        if niter >= max_iter:
            raise RuntimeError("no convergence")


def steady_state_temp(FF, E, rho, emiss, Fsurf=0.0, clamp=True):
    if E.ndim == 1:
        B = solve_radiosity(FF, E, rho)[0]
        if clamp:
            B = np.maximum(0, B)
        IR = FF @ ((1 - rho) * B + Fsurf)
        Q = solve_radiosity(FF, IR, 1)[0]
        if clamp:
            Q = np.maximum(0, Q)
        tot = (1 - rho) * B + emiss * Q + Fsurf
        if clamp:
            tot = np.maximum(0, tot)
        return (tot / (emiss * sigSB))**0.25
    B_arr = solve_radiosity(FF, E, rho)[0]
    T = []
    for B in B_arr.T:
        if clamp:
            B = np.maximum(0, B)
        IR = FF @ ((1 - rho) * B)
        Q = solve_radiosity(FF, IR, 1)[0]
        if clamp:
            Q = np.maximum(0, Q)
        T.append((((1 - rho) * B + emiss * Q) / (emiss * sigSB))**0.25)
    return np.array(T)
