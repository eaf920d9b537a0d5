"""Seeded synthetic workloads (host-side set-up, numpy).

There is no public dataset for this path: the workloads are generated from a
seed with the shapes, sizes and value distributions of the benchmark
configurations:

* ``tracer_transport`` - plain FP64 tracer transport on a 120 x 100 x 30 sigma
  grid, dx = dy = 1 km, Gaussian-smoothed random bathymetry 10-60 m with cells
  shallower than 12 m masked as land, solid-body rotation (max 0.5 m/s),
  w from continuity, a 3D Gaussian tracer blob, parabolic diffusivity
  1e-4..1e-2 m2/s; superbee, dt = 30 s.
* ``seamount`` - the baroclinic split-explicit box: 400 x 300 x 40 sigma,
  dx = 2 km, 4500 m deep with a 4000 m high, 25 km radius Gaussian seamount,
  T 20 -> 4 degC linear in depth, S = 35, f = 1e-4, 3D dt = 120 s with 30
  substeps.

Each returns a ``Workload`` with the host grid tree and initial fields as
numpy arrays (pygetm layout, halos included); the GPU path and the oracle are
both started from these same arrays.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, Optional

import numpy as np
from scipy.ndimage import gaussian_filter

from .domain import FILL_VALUE, HostGrid, calculate_sigma, create_cartesian


@dataclasses.dataclass
class Workload:
    name: str
    T: HostGrid
    dga: np.ndarray
    fields: Dict[str, np.ndarray]
    params: Dict[str, float]

    @property
    def cells(self) -> int:
        """Interior T cells, land included (the cell-update unit)."""
        return self.T.nx * self.T.ny * self.T.nz

    @property
    def wet_cells(self) -> int:
        return int((self.T.mask[self.T.interior[1:]] != 0).sum()) * self.T.nz


def _norm01(a):
    return (a - a.min()) / (a.max() - a.min())


def sigma_thicknesses(g: HostGrid, dga: np.ndarray, D: np.ndarray) -> np.ndarray:
    """Sigma.__call__ (python/pygetm/vertical_coordinates.py:106-113):
    hn = dga * D where mask != 0, FILL_VALUE elsewhere."""
    hn = np.full((dga.size,) + D.shape, FILL_VALUE)
    water = g.mask != 0
    hn[:, water] = dga[:, None] * D[water][None, :]
    return hn


def vertical_coordinates(g: HostGrid, hn: np.ndarray):
    """thickness2vertical_coordinates (python/src/wrapper.F90:409-426) in numpy,
    for set-up only (zc, zf start at -H as in python/pygetm/core.py:356-362)."""
    nz = hn.shape[0]
    zc = np.broadcast_to(-g.H_unmasked, hn.shape).copy()
    zf = np.broadcast_to(-g.H_unmasked, (nz + 1,) + hn.shape[1:]).copy()
    water = g.mask != 0
    H = g.H
    zf[0, water] = -H[water]
    for k in range(nz):
        zf[k + 1, water] = zf[k, water] + hn[k, water]
    zc[0, water] = -H[water] + 0.5 * hn[0, water]
    for k in range(1, nz):
        zc[k, water] = zc[k - 1, water] + 0.5 * (hn[k - 1, water] + hn[k, water])
    return zc, zf


def continuity_w(T: HostGrid, pk: np.ndarray, qk: np.ndarray) -> np.ndarray:
    """w from discrete continuity with ho == hn: the recursion of
    c_w_momentum_3d (python/src/momentum.F90:191-216) over the range pygetm
    passes (python/_pygetm.pyx:454), in numpy."""
    nz = pk.shape[0]
    w = np.zeros((nz + 1, T.ny_, T.nx_))
    dyu, dxv = T.ugrid.dy, T.vgrid.dx
    j0, j1 = T.haloy, T.haloy + T.ny + 1
    i0, i1 = T.halox, T.halox + T.nx + 1
    sl = (slice(j0, j1), slice(i0, i1))
    slw = (slice(j0, j1), slice(i0 - 1, i1 - 1))
    sls = (slice(j0 - 1, j1 - 1), slice(i0, i1))
    wet = T.mask[sl] == 1
    for k in range(1, nz):
        div = (pk[k - 1][sl] * dyu[sl] - pk[k - 1][slw] * dyu[slw] + qk[k - 1][sl] * dxv[sl] - qk[k - 1][sls] * dxv[sls]) * T.iarea[sl]
        wk = w[k - 1][sl] - div
        w[k][sl] = np.where(wet, wk, w[k][sl])
    return w


def _bathymetry(rng, nx, ny, Hmin, Hmax, Hland, land_fraction, sigma=8.0):
    """Gaussian-smoothed noise scaled to [Hmin, Hmax]; a power law on the
    normalised field puts the requested fraction of cells below Hland."""
    q = _norm01(gaussian_filter(rng.standard_normal((ny, nx)), sigma=sigma))
    qland = (Hland - Hmin) / (Hmax - Hmin)
    qf = np.quantile(q, land_fraction)
    p = np.log(qland) / np.log(qf)
    return Hmin + (Hmax - Hmin) * q**p


def rotating_transport(T: HostGrid, omega: float, D0: float, Htaper: float, Hland: float):
    """Depth-integrated transport in solid-body rotation about the domain
    centre, from a streamfunction psi on X points:
    psi = -omega/2 r^2 D0 phi(H_X) * xmask, phi = min(1, ((H_X-Hland)/Htaper)^2)
    for H_X > Hland else 0.  U = -(psi_N - psi_S)/dy, V = (psi_E - psi_W)/dx is
    discretely non-divergent, with zero transport through every masked face."""
    X = T.xgrid
    xc = 0.5 * (T.x[T.interior[1:]].min() + T.x[T.interior[1:]].max())
    yc = 0.5 * (T.y[T.interior[1:]].min() + T.y[T.interior[1:]].max())
    with np.errstate(invalid="ignore"):
        HX = X.H_unmasked
        phi = np.clip((HX - Hland) / Htaper, 0.0, None) ** 2
        phi = np.minimum(phi, 1.0)
        r2 = (X.x - xc) ** 2 + (X.y - yc) ** 2
        psi = np.where(X.mask != 0, -0.5 * omega * r2 * D0 * phi, 0.0)
    psi = np.nan_to_num(psi)
    U = np.zeros((T.ny_, T.nx_))
    V = np.zeros((T.ny_, T.nx_))
    # U(i, j) lies between corners X(i+1, j) [south] and X(i+1, j+1) [north];
    # V(i, j) between X(i, j+1) [west] and X(i+1, j+1) [east] (X = T shifted
    # by one corner: X local i is the south-west corner of T local i).
    U[:, :] = -(psi[1:, 1:] - psi[:-1, 1:]) / T.ugrid.dy
    V[:, :] = (psi[1:, 1:] - psi[1:, :-1]) / T.vgrid.dx
    U[T.ugrid.mask == 0] = 0.0
    V[T.vgrid.mask == 0] = 0.0
    return U, V


def tracer_transport(nx: int = 120, ny: int = 100, nz: int = 30, seed: int = 1, dt: float = 30.0) -> Workload:
    """Plain FP64 tracer-transport workload (120 x 100 x 30 by default)."""
    rng = np.random.default_rng(seed)
    dx = 1000.0
    x = dx * (np.arange(nx) + 0.5)
    y = dx * (np.arange(ny) + 0.5)
    H = _bathymetry(rng, nx, ny, 10.0, 60.0, 12.0, 0.15)
    mask = (H >= 12.0).astype(int)
    dom = create_cartesian(x, y, mask=mask, H=H, f=0.0)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    dga = calculate_sigma(nz)
    U, V = T.ugrid, T.vgrid
    fields: Dict[str, np.ndarray] = {}
    for g, n in ((T, "T"), (U, "U"), (V, "V"), (T.xgrid, "X")):
        D = np.where(g.mask != 0, g.H, FILL_VALUE)
        fields[f"D_{n}"] = D
        fields[f"hn_{n}"] = sigma_thicknesses(g, dga, D)
    uwet = U.mask != 0
    vwet = V.mask != 0
    Ut, Vt = rotating_transport(T, 1.0, 30.0, 10.0, 12.0)
    with np.errstate(invalid="ignore", divide="ignore"):
        u2 = np.where(uwet, Ut / fields["D_U"], 0.0)
        v2 = np.where(vwet, Vt / fields["D_V"], 0.0)
    scale = 0.5 / max(np.abs(u2).max(), np.abs(v2).max())
    u2 *= scale
    v2 *= scale
    uk = np.broadcast_to(u2, (nz,) + u2.shape).copy()
    vk = np.broadcast_to(v2, (nz,) + v2.shape).copy()
    pk = uk * np.where(uwet, fields["hn_U"], 0.0)
    qk = vk * np.where(vwet, fields["hn_V"], 0.0)
    w = continuity_w(T, pk, qk)
    zc, zf = vertical_coordinates(T, fields["hn_T"])
    D = fields["D_T"]
    xc = 0.5 * (x[0] + x[-1])
    yc = 0.5 * (y[0] + y[-1])
    x0, y0 = xc + 25000.0, yc
    L = 10000.0
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        c = np.exp(-((T.x - x0) ** 2 + (T.y - y0) ** 2)[None] / L**2 - ((zc + 0.5 * D[None]) / (0.25 * D[None])) ** 2)
    c = np.where(T.mask[None] != 0, c, FILL_VALUE)
    # parabolic diffusivity at interfaces, s = height fraction above the bottom
    s = np.linspace(0.0, 1.0, nz + 1)[:, None, None]
    nuh = np.broadcast_to(1e-4 + (1e-2 - 1e-4) * 4 * s * (1 - s), (nz + 1, T.ny_, T.nx_)).copy()
    nuh[:, T.mask == 0] = FILL_VALUE
    fields.update(uk=uk, vk=vk, w=w, tracer=c, nuh=nuh, zc_T=zc, zf_T=zf)
    return Workload("tracer_transport", T, dga, fields, dict(dt=dt, umax=0.5, scheme=5, cnpar=1.0))


def seamount(nx: int = 400, ny: int = 300, nz: int = 40, seed: int = 2, dx: float = 2000.0,
             timestep: float = 4.0, split_factor: int = 30) -> Workload:
    """Baroclinic seamount box (400 x 300 x 40 by default): 4500 m deep with a
    4000 m high Gaussian seamount of radius 25 km at the centre, f = 1e-4,
    closed boundaries, no wind, prescribed num = nuh = 1e-4 m2/s, bottom
    roughness z0 = 0.755 m (drag coefficient 2.5e-3 at D = 4500 m with the
    log-law of python/src/momentum.F90:93), T = 4 + 16 (z + 4500)/4500 degC,
    S = 35.  The random seed is unused: the configuration is deterministic."""
    del seed
    x = dx * (np.arange(nx) - 0.5 * (nx - 1))
    y = dx * (np.arange(ny) - 0.5 * (ny - 1))
    r2 = x[None, :] ** 2 + y[:, None] ** 2
    H = 4500.0 - 4000.0 * np.exp(-r2 / 25000.0**2)
    kappa, cd = 0.4, 2.5e-3
    z0 = 0.5 * 4500.0 / (np.exp(kappa / np.sqrt(cd)) - 1.0)
    dom = create_cartesian(x, y, H=H, f=1e-4, z0=z0)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    dga = calculate_sigma(nz)
    params = dict(timestep=timestep, split_factor=split_factor, num=1e-4, nuh=1e-4, z0=z0, scheme=5)
    return Workload("seamount", T, dga, {}, params)


def seamount_temperature(zc: np.ndarray) -> np.ndarray:
    """Linear stratification 20 degC at the surface to 4 degC at 4500 m."""
    return 4.0 + 16.0 * (zc + 4500.0) / 4500.0


def ensemble_member(rng: np.random.Generator, nmin: int = 64, nmax: int = 256, nzmin: int = 20,
                    nzmax: int = 40, dx: float = 1000.0) -> Workload:
    """One domain of the batched ensemble: sides log-uniform in [nmin, nmax],
    nz log-uniform in [nzmin, nzmax], smoothed bathymetry 10-100 m, a 10-30 %
    land mask (quantile threshold of a second smoothed field), a temperature
    drop of 5-15 degC from surface to 100 m, wind stress uniform in
    [0, 0.2] Pa along x, 20-40 substeps per 3D step."""
    nx = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
    ny = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
    nz = int(round(np.exp(rng.uniform(np.log(nzmin), np.log(nzmax)))))
    H = 10.0 + 90.0 * _norm01(gaussian_filter(rng.standard_normal((ny, nx)), sigma=6))
    landf = rng.uniform(0.1, 0.3)
    q = gaussian_filter(rng.standard_normal((ny, nx)), sigma=8)
    mask = (q >= np.quantile(q, landf)).astype(int)
    x = dx * (np.arange(nx) + 0.5)
    y = dx * (np.arange(ny) + 0.5)
    kappa, cd = 0.4, 2.5e-3
    z0 = 0.5 * 50.0 / (np.exp(kappa / np.sqrt(cd)) - 1.0)
    dom = create_cartesian(x, y, mask=mask, H=H, f=1e-4, z0=z0)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    dga = calculate_sigma(nz)
    split = int(rng.integers(20, 41))
    params = dict(timestep=10.0, split_factor=split, num=1e-4, nuh=1e-4, z0=z0, scheme=5,
                  taux=float(rng.uniform(0.0, 0.2)), dT=float(rng.uniform(5.0, 15.0)), land=landf)
    return Workload(f"member{nx}x{ny}x{nz}", T, dga, {}, params)


def ensemble(n: int = 256, seed: int = 4, **kwargs):
    """The batched ensemble: n independent members (seeded)."""
    rng = np.random.default_rng(seed)
    return [ensemble_member(rng, **kwargs) for _ in range(n)]


def member_temperature(zc: np.ndarray, dT: float) -> np.ndarray:
    """Linear stratification: 20 degC at the surface, dT colder at 100 m."""
    return 20.0 + dT * zc / 100.0


def land_fraction(wl: Workload) -> float:
    m = wl.T.mask[wl.T.interior[1:]]
    return float((m == 0).mean())


def serving_requests(rate: float, duration: float, seed: int = 5, nmin: int = 64, nmax: int = 512,
                     nzmin: int = 20, nzmax: int = 40, steps=(10, 200), precision: str = "mixed"):
    """Poisson request stream: arrivals at ``rate`` per second over
    ``duration`` seconds; each request is an ensemble-type domain with sides
    log-uniform in [nmin, nmax] and nz in [nzmin, nzmax], asking for a
    uniform number of 3D steps in ``steps``.  Domains are generated at
    admission (``make_workload``); ``cells_hint`` is known up front."""
    from .serving import Request

    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    rid = 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        member_seed = int(rng.integers(0, 2**31 - 1))
        sub = np.random.default_rng(member_seed)
        # the domain's sizes are the first draws of its own generator
        nx = int(round(np.exp(sub.uniform(np.log(nmin), np.log(nmax)))))
        ny = int(round(np.exp(sub.uniform(np.log(nmin), np.log(nmax)))))
        nz = int(round(np.exp(sub.uniform(np.log(nzmin), np.log(nzmax)))))
        nsteps = int(rng.integers(steps[0], steps[1] + 1))

        def make(member_seed=member_seed):
            return ensemble_member(np.random.default_rng(member_seed), nmin=nmin, nmax=nmax, nzmin=nzmin,
                                   nzmax=nzmax)

        reqs.append(Request(rid, make, nsteps, t, precision, (nx + 4) * (ny + 4) * (nz + 1)))
        rid += 1
    return reqs


M2_PERIOD = 44712.0  # s (M2 tidal constituent)


def tidal_channel(nx: int = 60, ny: int = 30, nz: int = 8, dx: float = 2000.0, seed: int = 7,
                  amplitude: float = 1.0) -> Workload:
    """A channel with three open boundaries of different kinds: west Flather
    (elevation) forced by an M2 tide of ``amplitude`` metres, tracers zero
    gradient; east clamped elevation (the same tide, lagged by 30 degrees),
    tracers sponge; north Flather (transport) with zero prescribed values,
    tracers clamped; south coast closed.  Smoothed bathymetry 20-50 m,
    f = 1e-4, z0 giving a drag coefficient of 2.5e-3 at 30 m."""
    from .open_boundaries import CLAMPED, FLATHER_ELEV, FLATHER_TRANSPORT, SPONGE, ZERO_GRADIENT

    rng = np.random.default_rng(seed)
    H = 20.0 + 30.0 * _norm01(gaussian_filter(rng.standard_normal((ny, nx)), sigma=4))
    x = dx * (np.arange(nx) + 0.5)
    y = dx * (np.arange(ny) + 0.5)
    kappa, cd = 0.4, 2.5e-3
    z0 = 0.5 * 30.0 / (np.exp(kappa / np.sqrt(cd)) - 1.0)
    dom = create_cartesian(x, y, H=H, f=1e-4, z0=z0)
    ob = dom.open_boundaries
    ob.add_left_boundary("W", 0, 0, ny, FLATHER_ELEV, ZERO_GRADIENT)
    ob.add_right_boundary("E", nx - 1, 0, ny, CLAMPED, SPONGE)
    ob.add_top_boundary("N", ny - 1, 1, nx - 1, FLATHER_TRANSPORT, CLAMPED)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    omega = 2.0 * np.pi / M2_PERIOD
    amp = np.zeros(ob.np)
    phase = np.zeros(ob.np)
    for b in ob:
        if b.name in ("W", "E"):
            amp[b.start:b.stop] = amplitude
            phase[b.start:b.stop] = 0.0 if b.name == "W" else -np.pi / 6
    ob.set_tide(omega, amp, phase)
    dga = calculate_sigma(nz)
    params = dict(timestep=5.0, split_factor=10, num=1e-4, nuh=1e-4, z0=z0, scheme=5)
    return Workload("tidal_channel", T, dga, {}, params)


def _fractal(rng, ny, nx, slope=1.5):
    """Field with a power-law amplitude spectrum k^-slope and random phases
    (spectral synthesis), scaled to [0, 1]."""
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    k = np.sqrt(kx**2 + ky**2)
    k[0, 0] = np.inf
    amp = k ** (-slope)
    spec = amp * np.exp(2j * np.pi * rng.uniform(size=amp.shape))
    return _norm01(np.fft.irfft2(spec, s=(ny, nx)))


def _water_runs(line):
    """(start, stop) of the runs of True in a 1D boolean array."""
    runs, start = [], None
    for n, w in enumerate(line):
        if w and start is None:
            start = n
        elif not w and start is not None:
            runs.append((start, n))
            start = None
    if start is not None:
        runs.append((start, len(line)))
    return runs


def shelf_sea(nx: int = 1000, ny: int = 800, nz: int = 30, dx: float = 1500.0, seed: int = 3,
              ntracer: int = 20, umax: float = 1.2, tide: float = 1.0) -> Workload:
    """The many-tracer shelf sea (1000 x 800 x 30 by default, dx 1.5 km):
    fractal bathymetry (amplitude spectrum k^-1.5) mapped to 5-200 m, land
    where a smoothed random field exceeds its 65th percentile (~35 %), open
    boundaries on every water run of the west edge (Flather elevation with an
    M2 tide of ``tide`` metres; tracers zero gradient) and of the south edge
    (clamped elevation, the tide lagged 60 degrees; tracers sponge).  The
    initial depth-integrated flow comes from a streamfunction of 8 seeded
    Fourier modes on X points (zero on land, so the discrete flow is
    non-divergent with no flow through the coast), scaled to a largest speed
    of ``umax`` m/s.  ``params['tracers']`` holds the ``ntracer`` initial
    passive-tracer fields, log-uniform in [1e-3, 10] (smoothed)."""
    from .open_boundaries import CLAMPED, FLATHER_ELEV, SPONGE, ZERO_GRADIENT

    rng = np.random.default_rng(seed)
    H = 5.0 + 195.0 * _fractal(rng, ny, nx)
    q = gaussian_filter(rng.standard_normal((ny, nx)), sigma=8)
    mask = (q <= np.quantile(q, 0.65)).astype(int)
    x = dx * (np.arange(nx) + 0.5)
    y = dx * (np.arange(ny) + 0.5)
    kappa, cd = 0.4, 2.5e-3
    z0 = 0.5 * 50.0 / (np.exp(kappa / np.sqrt(cd)) - 1.0)
    dom = create_cartesian(x, y, mask=mask, H=H, f=1.2e-4, z0=z0)
    ob = dom.open_boundaries
    for n, (s, e) in enumerate(_water_runs(mask[:, 0] == 1)):
        ob.add_left_boundary(f"W{n}", 0, s, e, FLATHER_ELEV, ZERO_GRADIENT)
    for n, (s, e) in enumerate(_water_runs(mask[0, 1:] == 1)):
        ob.add_bottom_boundary(f"S{n}", 0, s + 1, e + 1, CLAMPED, SPONGE)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    omega = 2.0 * np.pi / M2_PERIOD
    phase = np.zeros(ob.np)
    for b in ob:
        if b.name.startswith("S"):
            phase[b.start:b.stop] = -np.pi / 3
    ob.set_tide(omega, tide, phase)
    # streamfunction on X points (ny_+1, nx_+1): 8 Fourier modes, zero at X
    # points that touch land (X mask 0)
    X = T.xgrid
    xs = np.where(X.mask != 0, X.x, 0.0)
    ys = np.where(X.mask != 0, X.y, 0.0)
    psi = np.zeros(X.mask.shape)
    Lx, Ly = nx * dx, ny * dx
    for _ in range(8):
        kx = 2 * np.pi * rng.integers(1, 6) / Lx
        ky = 2 * np.pi * rng.integers(1, 6) / Ly
        psi += rng.uniform(0.5, 1.0) * np.sin(kx * xs + ky * ys + rng.uniform(0, 2 * np.pi))
    psi[X.mask == 0] = 0.0
    U = np.zeros((T.ny_, T.nx_))
    V = np.zeros((T.ny_, T.nx_))
    # U(j, i) between X(j, i+1) [south] and X(j+1, i+1) [north]; V(j, i)
    # between X(j+1, i) [west] and X(j+1, i+1) [east]
    U[:, :] = -(psi[1:, 1:] - psi[:-1, 1:])
    V[:, :] = psi[1:, 1:] - psi[1:, :-1]
    U[T.ugrid.mask != 1] = 0.0
    V[T.vgrid.mask != 1] = 0.0
    speed = max(np.abs(U[T.ugrid.mask == 1] / T.ugrid.H[T.ugrid.mask == 1]).max(),
                np.abs(V[T.vgrid.mask == 1] / T.vgrid.H[T.vgrid.mask == 1]).max())
    U *= umax / speed
    V *= umax / speed
    tracers = []
    for _ in range(ntracer):
        f = 10.0 ** (-3.0 + 4.0 * _norm01(gaussian_filter(rng.uniform(size=(T.ny_, T.nx_)), sigma=4)))
        tracers.append(f)
    dga = calculate_sigma(nz)
    params = dict(timestep=10.0, split_factor=6, num=1e-4, nuh=1e-4, z0=z0, scheme=5, U=U, V=V, tracers=tracers)
    return Workload(f"shelf_sea {nx}x{ny}x{nz}", T, dga, {}, params)


def start_shelf_sea(wl: Workload, precision: str = "mixed", device="cuda"):
    """A BAROTROPIC_3D simulation of ``shelf_sea`` with its passive tracers,
    initial flow (uniform over depth) and tide, started."""
    import torch

    from .simulation import RunType, Simulation

    p = wl.params
    sim = Simulation(wl.T, wl.dga, runtype=RunType.BAROTROPIC_3D, num=p["num"], nuh=p["nuh"], precision=precision,
                     device=device)
    trs = [sim.tracers.add(f"tracer{n:02d}") for n in range(len(p["tracers"]))]
    for tr, f in zip(trs, p["tracers"]):
        tr.all_values.copy_(torch.from_numpy(np.broadcast_to(f, tr.all_values.shape).copy()))
    m = sim.momentum
    for tp2, tp3, g in ((m.U, m.pk, sim.U), (m.V, m.qk, sim.V)):
        src = torch.from_numpy(p["U"] if tp2 is m.U else p["V"]).to(tp2.all_values)
        tp2.all_values.copy_(src)
        frac = torch.where(g.D.all_values > 0, g.hn.all_values / g.D.all_values, torch.zeros_like(g.hn.all_values))
        tp3.all_values.copy_((src * frac).to(tp3.all_values.dtype))
    sim.start(p["timestep"], p["split_factor"])
    return sim
