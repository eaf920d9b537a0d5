"""Shared set-up for the tests: small domains built with the same host-side
code the GPU path uses, in oracle (numpy) form and device form."""

from __future__ import annotations

import numpy as np

from getm_gb300.domain import FILL_VALUE, calculate_sigma, create_cartesian


def rel_err(a, b, where=None):
    """max |a - b| / max |b| over the selected points."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    if where is not None:
        a = a[..., where]
        b = b[..., where]
    scale = np.abs(b).max()
    if scale == 0:
        scale = 1.0
    return float(np.abs(a - b).max() / scale)


def column_grid(nx=50, ny=52, nz=25, ddu=0.0, ddl=0.0, seed=0, H=50.0, land=0.5):
    """Domain of python/tests/test_vertical_diffusion.py:21-43: 50 km square,
    H = 50 m, a random land mask, sigma layers, ho = hn."""
    rng = np.random.default_rng(seed)
    EXTENT = 50000.0
    dom = create_cartesian(np.linspace(0, EXTENT, nx), np.linspace(0, EXTENT, ny), f=0.0, H=H)
    dom.mask = rng.random((ny, nx)) > land
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=0)
    dga = calculate_sigma(nz, ddl=ddl, ddu=ddu)
    hn = np.full((nz, T.ny_, T.nx_), FILL_VALUE)
    water = T.mask != 0
    hn[:, water] = dga[:, None] * T.H[water][None, :]
    return T, dga, hn


def full_grid(nx=40, ny=30, nz=10, seed=0, land=0.15, dx=1000.0, Hmin=10.0, Hmax=40.0, f=0.0, velocity_grids=2):
    """Random-bathymetry domain with land, all eight staggered grids."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    q = gaussian_filter(rng.standard_normal((ny, nx)), 3)
    q = (q - q.min()) / (q.max() - q.min())
    H = Hmin + (Hmax - Hmin) * q
    mask = (q >= np.quantile(q, land)).astype(int)
    x = dx * (np.arange(nx) + 0.5)
    y = dx * (np.arange(ny) + 0.5)
    dom = create_cartesian(x, y, mask=mask, H=H, f=f)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=velocity_grids)
    return T, rng
