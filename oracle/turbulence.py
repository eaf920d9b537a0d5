"""CPU restatement of the k-epsilon closure - TEST INFRASTRUCTURE ONLY.

The reference takes num and nuh from GOTM through pygotm
(python/pygetm/vertical_mixing.py:60-188; advanced at
python/pygetm/simulation.py:1107-1115).  GOTM is not vendored, so this is a
restatement of the published model the library implements (the
buoyancy-extended k-epsilon model of Rodi 1987 with constant stability
functions, log-law boundary values, Galperin et al. 1988 length-scale
limitation, Patankar 1980 source linearisation), with the same operation
order, vectorised over the water columns.  Parity against GOTM itself is
unpinned.
"""

from __future__ import annotations

import numpy as np

DEFAULTS = dict(cm0=0.5477, kappa=0.4, sig_k=1.0, sig_e=1.3, c1=1.44, c2=1.92, c3_minus=-0.4, c3_plus=1.0,
                galp=0.53, prandtl=1.0, k_min=1e-10, eps_min=1e-12)


def _wall(p, ustar, z0):
    cm0 = p["cm0"]
    k = np.maximum(ustar * ustar / (cm0 * cm0), p["k_min"])
    e = np.maximum(cm0 * cm0 * cm0 * k * np.sqrt(k) / (p["kappa"] * z0), p["eps_min"])
    return k, e


def _solve(x, h, x0, xn, K, Q, S, dt):
    """Implicit diffusion-source update of interfaces 1..nz-1 of every
    column (x: (nz+1, ncol), h: (nz, ncol); K: (nz, ncol) at the layers;
    Q, S: (nz+1, ncol) sources, rows 1..nz-1 used); Dirichlet x0, xn."""
    nz = h.shape[0]
    cp = np.zeros_like(x)
    dp = np.zeros_like(x)
    cprev = np.zeros_like(x0)
    dprev = x0.copy()
    hb, Kb = h[0], K[0]
    for i in range(1, nz):
        ht, Kt = h[i], K[i]
        dz = 0.5 * (hb + ht)
        lo = -dt * Kb / hb
        up = -dt * Kt / ht
        b = dz - lo - up - dt * dz * S[i]
        d = dz * (x[i] + dt * Q[i])
        if i == nz - 1:
            d = d - up * xn
        den = b - lo * cprev
        cprev = up / den
        dprev = (d - lo * dprev) / den
        cp[i] = cprev
        dp[i] = dprev
        hb, Kb = ht, Kt
    out = x.copy()
    xv = xn
    for i in range(nz - 1, 0, -1):
        xv = dp[i] - cp[i] * xv
        out[i] = xv
    out[0] = x0
    out[nz] = xn
    return out


def keps_advance(T, timestep, h, ustar_s, ustar_b, z0s, z0b, NN, SS, tke, eps, L, num, nuh, params=None):
    """Advance tke, eps, L, num, nuh (in place; (nz+1, ny_, nx_) arrays) on
    the interior water columns (mask == 1) of grid T."""
    p = dict(DEFAULTS, **(params or {}))
    nz = h.shape[0]
    sel = np.zeros(T.mask.shape, dtype=bool)
    sel[T.haloy:T.ny_ - T.haloy, T.halox:T.nx_ - T.halox] = True
    sel &= T.mask == 1
    hh = h[:, sel]
    k0, e0, nu0, nh0 = tke[:, sel], eps[:, sel], num[:, sel], nuh[:, sel]
    N2, S2 = NN[:, sel], SS[:, sel]
    cmu = p["cm0"] * p["cm0"] * p["cm0"] * p["cm0"]
    cde = p["cm0"] * p["cm0"] * p["cm0"]
    kb, eb = _wall(p, ustar_b[sel], z0b[sel])
    ks, es = _wall(p, ustar_s[sel], z0s[sel])
    prod = nu0 * S2
    buoy = -nh0 * N2
    with np.errstate(divide="ignore", invalid="ignore"):
        pos = prod + buoy > 0.0
        Qk = np.where(pos, prod + buoy, prod)
        Sk = np.where(pos, -e0 / k0, -(e0 - buoy) / k0)
        Kk = 0.5 * (nu0[:-1] + nu0[1:]) / p["sig_k"]
        k1 = _solve(k0, hh, kb, ks, Kk, Qk, Sk, timestep)
        k1[1:nz] = np.maximum(k1[1:nz], p["k_min"])
        r = e0 / k1
        c3 = np.where(buoy > 0.0, p["c3_plus"], p["c3_minus"])
        Qe = r * (p["c1"] * prod + c3 * buoy)
        Se = -p["c2"] * r
        Ke = 0.5 * (nu0[:-1] + nu0[1:]) / p["sig_e"]
        e1 = _solve(e0, hh, eb, es, Ke, Qe, Se, timestep)
        e1 = np.maximum(e1, p["eps_min"])
        lmax = p["galp"] * np.sqrt(2.0 * k1 / N2)
        lim = np.maximum(e1, cde * k1 * np.sqrt(k1) / lmax)
        inner = np.zeros_like(e1, dtype=bool)
        inner[1:nz] = True
        e1 = np.where(inner & (N2 > 0.0), lim, e1)
    tke[:, sel] = k1
    eps[:, sel] = e1
    L[:, sel] = cde * k1 * np.sqrt(k1) / e1
    nu = cmu * k1 * k1 / e1
    num[:, sel] = nu
    nuh[:, sel] = nu / p["prandtl"]


def initial_state(nz, shape, params=None):
    """GOTM-style initial turbulence: k = k_min, eps = eps_min, L, num and
    nuh from them (arrays of (nz + 1,) + shape)."""
    p = dict(DEFAULTS, **(params or {}))
    k = np.full((nz + 1,) + shape, p["k_min"])
    e = np.full((nz + 1,) + shape, p["eps_min"])
    cde = p["cm0"] * p["cm0"] * p["cm0"]
    cmu = p["cm0"] * p["cm0"] * p["cm0"] * p["cm0"]
    L = cde * k * np.sqrt(k) / e
    num = cmu * k * k / e
    return k, e, L, num, num / p["prandtl"]
