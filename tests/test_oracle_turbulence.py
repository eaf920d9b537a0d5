"""The k-epsilon closure's CPU restatement against properties of the model
(no reference output exists: GOTM is external to the reference, so parity
with it is unpinned): decay of homogeneous turbulence as the analytic
solution of dk/dt = -eps, deps/dt = -c2 eps^2/k; positivity and the lower
limits; the Galperin length-scale bound in stable stratification;
consistency of num, nuh and L with k and eps."""

import numpy as np
import pytest

from oracle import turbulence as K


class _Grid:
    def __init__(self, ny, nx, halo=2):
        self.nx_, self.ny_, self.halox, self.haloy = nx, ny, halo, halo
        self.mask = np.ones((ny, nx), dtype=np.int32)


def _columns(nz=40, ny=6, nx=7, H=400.0):
    T = _Grid(ny, nx)
    h = np.full((nz, ny, nx), H / nz)
    z2 = np.zeros((ny, nx))
    return T, h, z2


def test_homogeneous_decay_follows_the_analytic_law():
    """Without shear, stratification or wall stress, interior turbulence far
    from the walls decays as k(t) = k0 (1 + (c2 - 1) eps0 t / k0)^(-1/(c2-1))."""
    T, h, z2 = _columns()
    nz = h.shape[0]
    p = K.DEFAULTS
    k0, e0 = 1e-4, 1e-7
    tke = np.full((nz + 1,) + z2.shape, k0)
    eps = np.full_like(tke, e0)
    L = np.zeros_like(tke)
    cmu = p["cm0"] ** 4
    num = np.full_like(tke, cmu * k0 * k0 / e0)
    nuh = num.copy()
    zero = np.zeros_like(tke)
    dt, n = 10.0, 100
    for _ in range(n):
        K.keps_advance(T, dt, h, z2 + 0.0, z2 + 0.0, z2 + 0.1, z2 + 0.01, zero, zero, tke, eps, L, num, nuh)
    t = dt * n
    c2 = p["c2"]
    k_exact = k0 * (1.0 + (c2 - 1.0) * e0 * t / k0) ** (-1.0 / (c2 - 1.0))
    k_mid = tke[nz // 2, 3, 3]
    assert k_mid == pytest.approx(k_exact, rel=0.02)
    assert k_mid < k0


def test_positivity_limits_and_consistency():
    rng = np.random.default_rng(3)
    T, h, z2 = _columns(nz=25)
    nz = h.shape[0]
    p = K.DEFAULTS
    shape = (nz + 1,) + z2.shape
    tke, eps, L, num, nuh = K.initial_state(nz, z2.shape)
    NN = rng.uniform(-1e-5, 1e-4, shape)
    SS = rng.uniform(0.0, 1e-4, shape)
    us = rng.uniform(0.0, 0.02, z2.shape)
    ub = rng.uniform(0.0, 0.02, z2.shape)
    for _ in range(20):
        K.keps_advance(T, 60.0, h, us, ub, z2 + 0.1, z2 + 0.005, NN, SS, tke, eps, L, num, nuh)
    sel = (slice(None), slice(2, -2), slice(2, -2))
    assert (tke[sel] >= p["k_min"]).all() and (eps[sel] >= p["eps_min"]).all()
    assert np.isfinite(num[sel]).all() and (num[sel] > 0).all()
    cm0 = p["cm0"]
    np.testing.assert_allclose(num[sel], cm0 ** 4 * tke[sel] ** 2 / eps[sel], rtol=1e-12)
    np.testing.assert_allclose(nuh[sel], num[sel] / p["prandtl"], rtol=1e-15)
    np.testing.assert_allclose(L[sel], cm0 ** 3 * tke[sel] ** 1.5 / eps[sel], rtol=1e-12)
    # Galperin: L <= 0.53 sqrt(2 k / N2) at interior interfaces with N2 > 0
    inner = (slice(1, nz), slice(2, -2), slice(2, -2))
    stable = NN[inner] > 0
    lmax = p["galp"] * np.sqrt(2.0 * tke[inner][stable] / NN[inner][stable])
    assert (L[inner][stable] <= lmax * (1 + 1e-12)).all()
    # log-law values at the walls
    kb = np.maximum(ub ** 2 / cm0 ** 2, p["k_min"])
    np.testing.assert_allclose(tke[0][2:-2, 2:-2], kb[2:-2, 2:-2], rtol=1e-15)


def test_stratification_suppresses_mixing():
    """The same shear on developed turbulence (k = 1e-4 m2 s-2, eps = 1e-7
    m2 s-3, where shear production exceeds dissipation) with and without
    stable stratification: buoyancy destruction leaves far less viscosity.
    (From the minimum state k_min, eps_min this shear could not grow
    turbulence at all: k-epsilon needs SS > eps^2 / (cmu k^2) for that.)"""
    T, h, z2 = _columns(nz=30)
    nz = h.shape[0]
    shape = (nz + 1,) + z2.shape
    out = {}
    cmu = K.DEFAULTS["cm0"] ** 4
    for n2 in (0.0, 1e-4):
        tke = np.full(shape, 1e-4)
        eps = np.full(shape, 1e-7)
        L = np.zeros(shape)
        num = cmu * tke * tke / eps
        nuh = num.copy()
        NN = np.full(shape, n2)
        SS = np.full(shape, 1e-4)
        for _ in range(200):
            K.keps_advance(T, 30.0, h, z2 + 0.01, z2 + 0.01, z2 + 0.1, z2 + 0.005, NN, SS, tke, eps, L, num, nuh)
        out[n2] = num[nz // 2, 3, 3]
    assert out[1e-4] < 0.5 * out[0.0]


def test_simulation_with_closure_open_boundaries():
    """The oracle split-explicit step of a tidal channel with the closure: the
    viscosity at each open-boundary point is its inward neighbour's
    (zero gradient, python/pygetm/vertical_mixing.py:120,186), and the
    turbulence stays finite and positive."""
    from getm_gb300 import workloads
    from oracle.models import Simulation as OS

    wl = workloads.tidal_channel(nx=24, ny=16, nz=5)
    p = wl.params
    o = OS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], taux=0.2, keps={})
    o.start(p["timestep"], p["split_factor"])
    for _ in range(3 * p["split_factor"]):
        o.advance()
    ob = wl.T.open_boundaries
    on_boundary = set(zip(ob.j.tolist(), ob.i.tolist()))
    checked = 0
    for q in range(ob.np):  # (a point whose neighbour is a boundary point can change after its own update)
        jj, ii = ob.j[q] + ob.dj[q], ob.i[q] + ob.di[q]
        if (jj, ii) not in on_boundary:
            np.testing.assert_array_equal(o.num[:, ob.j[q], ob.i[q]], o.num[:, jj, ii])
            checked += 1
    assert checked > ob.np - 4
    wet = o.T.mask == 1
    assert np.isfinite(o.tke[:, wet]).all() and (o.tke[:, wet] > 0).all() and (o.num[:, wet] > 0).all()
