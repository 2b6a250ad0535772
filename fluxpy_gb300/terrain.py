"""Synthetic meshes for the benchmark workloads (seeded, no data files).

* ``spherical_crater``: the square [-1, 1]^2 with a spherical bowl of
  diameter 1 and depth/diameter 0.2, triangulated by Delaunay from 2,000
  uniform random points (numpy default_rng(0)) plus the boundary points of a
  40 x 40 grid (~4.3k triangles), normals up.
* ``fbm_terrain``: an n x n fractional-Brownian height field (spectral
  synthesis, Hurst exponent H, rescaled to a target RMS slope) with
  power-law craters of depth/diameter 0.2 added, on a regular grid of unit
  spacing triangulated into 2 (n-1)^2 facets (n = 512: 522,242 facets).
* ``sun_directions``: unit vectors from elevation/azimuth in degrees.

These stand in for the reference's example inputs (DEMs, SPICE kernels),
which are not distributed with it.
"""
from __future__ import annotations

import numpy as np


def _orient_up(V, F):
    e1 = V[F[:, 1]] - V[F[:, 0]]
    e2 = V[F[:, 2]] - V[F[:, 0]]
    nz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    F = F.copy()
    flip = nz < 0
    F[flip] = F[flip][:, [0, 2, 1]]
    return F


def spherical_crater(n_points=2000, seed=0, boundary_grid=40, diameter=1.0, depth_ratio=0.2):
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-1.0, 1.0, size=(n_points, 2))
    g = np.linspace(-1.0, 1.0, boundary_grid)
    edge = [np.column_stack([g, np.full_like(g, -1.0)]), np.column_stack([g, np.full_like(g, 1.0)]),
            np.column_stack([np.full(g.size - 2, -1.0), g[1:-1]]),
            np.column_stack([np.full(g.size - 2, 1.0), g[1:-1]])]
    xy = np.vstack([pts] + edge)
    tri = Delaunay(xy)
    F = tri.simplices.astype(np.int64)
    rc = diameter / 2
    d = depth_ratio * diameter
    Rs = (rc**2 + d**2) / (2 * d)
    r = np.sqrt((xy**2).sum(1))
    z = np.where(r < rc, (Rs - d) - np.sqrt(np.maximum(Rs**2 - r**2, 0.0)), 0.0)
    V = np.column_stack([xy, z]).astype(np.float64)
    return V, _orient_up(V, F)


def _fbm_heights(n, hurst, rng):
    kx = np.fft.fftfreq(n)
    ky = np.fft.fftfreq(n)
    k = np.sqrt(kx[:, None]**2 + ky[None, :]**2)
    k[0, 0] = 1.0
    amp = k**(-(hurst + 1.0))
    amp[0, 0] = 0.0
    phase = rng.uniform(0, 2 * np.pi, size=(n, n))
    noise = rng.standard_normal((n, n))
    spec = amp * noise * np.exp(1j * phase)
    return np.real(np.fft.ifft2(spec))


def _add_craters(Z, n_craters, rng, depth_ratio=0.2, dmin=8.0, dmax=None, slope=-2.0):
    n = Z.shape[0]
    dmax = dmax or n / 4
    # cumulative size-frequency N(>D) ~ D^slope: inverse-CDF sampling
    u = rng.uniform(size=n_craters)
    a, b = dmin**slope, dmax**slope
    D = (a + u * (b - a))**(1.0 / slope)
    cx = rng.uniform(0, n - 1, n_craters)
    cy = rng.uniform(0, n - 1, n_craters)
    yy, xx = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    for di, x0, y0 in zip(D, cx, cy):
        rc = di / 2
        d = depth_ratio * di
        Rs = (rc**2 + d**2) / (2 * d)
        r2 = (xx - x0)**2 + (yy - y0)**2
        inside = r2 < rc**2
        bowl = (Rs - d) - np.sqrt(np.maximum(Rs**2 - r2, 0.0))
        Z[inside] += bowl[inside]
        # a low raised rim decaying outside the bowl
        ring = (~inside) & (r2 < (1.5 * rc)**2)
        rr = np.sqrt(r2[ring])
        Z[ring] += 0.04 * di * np.cos(np.pi / 2 * (rr - rc) / (0.5 * rc))**2
    return Z


def fbm_terrain(n=512, hurst=0.8, rms_slope_deg=20.0, seed=1, n_craters=30, spacing=1.0):
    rng = np.random.default_rng(seed)
    Z = _fbm_heights(n, hurst, rng)
    gy, gx = np.gradient(Z, spacing)
    rms = np.sqrt(np.mean(gx**2 + gy**2))
    Z *= np.tan(np.deg2rad(rms_slope_deg)) / rms
    Z = _add_craters(Z, n_craters, rng)
    yy, xx = np.meshgrid(np.arange(n) * spacing, np.arange(n) * spacing, indexing="ij")
    V = np.column_stack([xx.ravel(), yy.ravel(), Z.ravel()]).astype(np.float64)
    idx = np.arange(n * n).reshape(n, n)
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, :-1].ravel()
    d = idx[1:, 1:].ravel()
    F = np.vstack([np.column_stack([a, b, d]), np.column_stack([a, d, c])]).astype(np.int64)
    # interleave the two triangles of each grid cell so that facet order is
    # spatially coherent
    F = F.reshape(2, -1, 3).transpose(1, 0, 2).reshape(-1, 3)
    return V, _orient_up(V, F)


def sun_directions(elev_deg, azim_deg):
    e = np.deg2rad(np.atleast_1d(elev_deg))
    a = np.deg2rad(np.atleast_1d(azim_deg))
    return np.column_stack([np.cos(e) * np.cos(a), np.cos(e) * np.sin(a), np.sin(e)])


def random_sun_directions(K=1024, seed=2, elev=(1.0, 30.0)):
    rng = np.random.default_rng(seed)
    return sun_directions(rng.uniform(*elev, K), rng.uniform(0.0, 360.0, K))
