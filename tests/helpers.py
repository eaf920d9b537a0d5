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


def _random_closed_domain(nx, ny, nz, seed, dx):
    """Smoothed random bathymetry (20-100 m) and a land mask (15 %) of a
    closed domain, and a builder of its host grid tree."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)

    def n01(a):
        return (a - a.min()) / (a.max() - a.min())

    H = 20.0 + 80.0 * n01(gaussian_filter(rng.standard_normal((ny, nx)), 3))
    q = gaussian_filter(rng.standard_normal((ny, nx)), 3)
    mask = (q > np.quantile(q, 0.15)).astype(int)
    z0 = 0.5 * 50.0 / (np.exp(0.4 / np.sqrt(2.5e-3)) - 1.0)

    def make(H, mask, f=1e-4):
        ny_, nx_ = H.shape
        dom = create_cartesian(dx * (np.arange(nx_) + 0.5), dx * (np.arange(ny_) + 0.5), mask=mask, H=H, f=f,
                               z0=z0)
        return dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)

    return H, mask, make


def rotated_pair(nx=24, ny=18, nz=6, seed=3, dx=2000.0):
    """A closed domain with smoothed random bathymetry and land, and the same
    domain rotated by 90 degrees (arrays A.T[::-1]), as in
    python/tests/test_rotation.py (Domain.rotate): host grid trees (original,
    rotated) and the sigma fractions."""
    H, mask, make = _random_closed_domain(nx, ny, nz, seed, dx)
    return make(H, mask), make(rot2(H), rot2(mask)), calculate_sigma(nz)


def mirrored_pair(nx=24, ny=18, nz=6, seed=3, dx=2000.0, f=1e-4):
    """The same closed domain and its mirror image in y (arrays A[::-1]); the
    mirror image of a flow on an f-plane is a flow on the f-plane of -f, so
    the mirrored domain gets -f."""
    H, mask, make = _random_closed_domain(nx, ny, nz, seed, dx)
    return make(H, mask, f), make(H[::-1], mask[::-1], -f), calculate_sigma(nz)


def mirror_errors(orig, mir, masks):
    """Relative errors of the mirrored run against the original run mirrored
    in y: T and U points map row to row (A[..., ::-1, :]); V points (between
    rows) at row p come from -V at row NY-2-p (the last row has no
    counterpart)."""
    mT, mU, mV = (m == 1 for m in masks)
    mV = mV.copy()
    mV[-1, :] = False

    def rel(a, b, m):
        a, b = a[..., m], b[..., m]
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    def flip(a):
        return a[..., ::-1, :]

    def shifted(a):
        out = np.zeros_like(a)
        out[..., :-1, :] = -flip(a)[..., 1:, :]
        return out

    return {"z": rel(mir["z"], flip(orig["z"]), mT), "temp": rel(mir["temp"], flip(orig["temp"]), mT),
            "U": rel(mir["U"], flip(orig["U"]), mU), "uk": rel(mir["uk"], flip(orig["uk"]), mU),
            "V": rel(mir["V"], shifted(orig["V"]), mV), "vk": rel(mir["vk"], shifted(orig["vk"]), mV)}


def rot2(a):
    """A 2D array of T points (or of V points, see rotation_errors) rotated
    with its domain."""
    return a.T[::-1, :]


def rot3(a):
    return a.transpose(0, 2, 1)[:, ::-1, :]


def rotation_errors(orig, rot, masks):
    """Relative errors of the rotated run against the original run rotated:
    ``orig``/``rot`` map z, temp, U, V, uk, vk to arrays (numpy) of each run,
    ``masks`` the rotated domain's T, U and V masks.  Under the rotation
    x_rot = y and y_rot = -x, so U_rot = V rotated, and V_rot at row p is -U
    at the original column NX-2-p (the last row has no counterpart)."""
    mT, mU, mV = (m == 1 for m in masks)
    mV = mV.copy()
    mV[-1, :] = False

    def rel(a, b, m):
        a, b = a[..., m], b[..., m]
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    def shifted(a):  # -U rotated and shifted by one row (V_rot points)
        out = np.zeros(a.shape[:-2] + a.shape[-1:] + a.shape[-2:-1])
        r = rot2(a) if a.ndim == 2 else rot3(a)
        out[..., :-1, :] = -r[..., 1:, :]
        return out

    return {"z": rel(rot["z"], rot2(orig["z"]), mT), "temp": rel(rot["temp"], rot3(orig["temp"]), mT),
            "U": rel(rot["U"], rot2(orig["V"]), mU), "uk": rel(rot["uk"], rot3(orig["vk"]), mU),
            "V": rel(rot["V"], shifted(orig["U"]), mV), "vk": rel(rot["vk"], shifted(orig["uk"]), mV)}
