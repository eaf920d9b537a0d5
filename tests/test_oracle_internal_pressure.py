"""Pins the oracle's internal-pressure restatements (Blumberg-Mellor and
Shchepetkin-McWilliams) against the analytic cases of
python/tests/test_internal_pressure.py:21-93: a lock exchange gives
dP/dx = -zc g (rho_max - rho_min)/dx at the front, a linear density gives a
horizontally uniform gradient, and the cross-front component is exactly 0."""

import numpy as np
import pytest

from getm_gb300.domain import calculate_sigma, create_cartesian
from getm_gb300.workloads import sigma_thicknesses
from oracle import oracle as O

GRAVITY = 9.81
RHO0 = 1025.0


def _grids(ddu, H=100.0, nz=30):
    x = np.linspace(0, 50000, 101)
    y = np.linspace(0, 100000, 100)
    dom = create_cartesian(x, y, interfaces=True, f=0.0, H=H)
    Th = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=1)
    dga = calculate_sigma(nz, ddu=ddu)
    T = O.make_grids(Th)
    for g in (T, T.ugrid, T.vgrid):
        D = np.where(g.mask != 0, g.H, g.D)
        g.D[...] = D
        g.hn[...] = sigma_thicknesses(g.host, dga, D)
        O.thickness2vertical_coordinates(g, g.H, g.hn, g.zc, g.zf)
    zin = np.zeros((T.ny_, T.nx_))
    return T, zin


def _run(method, T, zin, buoy):
    U, V = T.ugrid, T.vgrid
    idpdx = np.zeros((T.nz, U.ny_, U.nx_))
    idpdy = np.zeros((T.nz, V.ny_, V.nx_))
    if method == "bm":
        O.blumberg_mellor(T, buoy, idpdx, idpdy)
    else:
        O.shchepetkin_mcwilliams(T, buoy, idpdx, idpdy, zin)
    return idpdx, idpdy


@pytest.mark.parametrize("method", ["bm", "smcw"])
@pytest.mark.parametrize("ddu", [0.0, 1.0, 2.0])
def test_lock_exchange_and_linear_density(method, ddu):
    rho_min, rho_max = 1020.0, 1025.0
    T, zin = _grids(ddu)
    U, V = T.ugrid, T.vgrid
    it = T.interior
    wetU = np.isin(U.mask, (1, 2))[U.interior[1:]]
    wetV = np.isin(V.mask, (1, 2))[V.interior[1:]]
    tol = 1e-14

    # lock exchange in x
    rho = np.full((T.nz, T.ny_, T.nx_), RHO0)
    rho[it][:, :, :50] = rho_min
    rho[it][:, :, 50:] = rho_max
    buoy = (-GRAVITY / RHO0) * (rho - RHO0)
    idpdx, idpdy = _run(method, T, zin, buoy)
    assert (idpdy[U.interior][:, wetV] == 0.0).all() if wetV.any() else True
    dP_dx = -U.zc[U.interior][:, 0, 0] * GRAVITY * (rho_max - rho_min) / U.dx[U.interior[1:]][0, 0]
    dU = (-dP_dx / RHO0) * U.hn[U.interior][:, 0, 0]
    assert np.abs(dU - idpdx[U.interior][:, 0, 49]).max() < tol

    # linear density in x: uniform gradient
    rho[it] = rho_min + (rho_max - rho_min) * T.x[it[1:]] / 100000
    buoy = (-GRAVITY / RHO0) * (rho - RHO0)
    idpdx, idpdy = _run(method, T, zin, buoy)
    vals = idpdx[U.interior][:, 0, :][:, wetU[0]]
    assert np.abs(vals - vals[:, :1]).max() < tol

    # lock exchange in y
    rho = np.full((T.nz, T.ny_, T.nx_), RHO0)
    rho[it][:, :50, :] = rho_min
    rho[it][:, 50:, :] = rho_max
    buoy = (-GRAVITY / RHO0) * (rho - RHO0)
    idpdx, idpdy = _run(method, T, zin, buoy)
    assert (idpdx[U.interior][:, wetU] == 0.0).all()
    dP_dy = -V.zc[V.interior][:, 0, 0] * GRAVITY * (rho_max - rho_min) / V.dy[V.interior[1:]][0, 0]
    dV = (-dP_dy / RHO0) * V.hn[V.interior][:, 0, 0]
    assert np.abs(dV - idpdy[V.interior][:, 49, 0]).max() < tol
