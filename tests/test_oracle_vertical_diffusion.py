"""Pins the oracle's vertical diffusion against the known-answer and invariant
tests of python/tests/test_vertical_diffusion.py:67-275 (column conservation,
no horizontal variability, bounds, the analytic relative source 1/(1-r)^N)."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import column_grid

DT = 600.0
NSTEP = 100
GRIDS = [dict(), dict(ddu=1.0), dict(ddl=1.0)]
CNPARS = [0.5, 0.75, 1.0]


def _setup(grid_args, seed=0):
    Th, dga, hn = column_grid(seed=seed, **grid_args)
    T = O.make_grids(Th)
    T.hn[...] = hn
    T.ho[...] = hn
    return T


def _diffuse(T, tracer_in, nuh, cnpar, tolerance=1e-13, sources=None, change_ho=False, rng=None):
    """python/tests/test_vertical_diffusion.py:67-146"""
    wet = T.mask == 1
    tracer = tracer_in.copy()
    vdif = O.VerticalDiffusion(T, cnpar=cnpar)
    nuh = nuh.copy()
    nuh[:, ~wet] = np.nan
    nuh[0] = np.nan
    nuh[-1] = np.nan
    interior = T.interior
    expected = (tracer_in * T.hn)[:, wet].sum(axis=0)
    for _ in range(NSTEP):
        if change_ho:
            T.ho[...] = T.hn
            pert = rng.lognormal(np.log(T.hn[:, wet].mean(axis=1)), 0.1)
            T.hn[:, wet] = pert[:, None]
        vdif(nuh, DT, tracer, ea4=sources, use_ho=change_ho)
    vals = tracer[:, wet]
    assert np.isfinite(vals).all()
    col_range = vals.max(axis=1) - vals.min(axis=1)
    assert col_range.max() == 0.0, "horizontal variability after diffusion"
    if sources is None and not change_ho:
        ini = tracer_in[:, wet]
        eps = tolerance * max(abs(vals.min()), abs(vals.max()))
        assert vals.max() <= ini.max() + eps
        assert vals.min() >= ini.min() - eps
    if sources is not None:
        expected = expected + sources[:, wet].sum(axis=0) * NSTEP
    integral = (tracer * T.hn)[:, wet].sum(axis=0)
    rel = np.abs(integral - expected).max() / np.abs(expected).max()
    assert rel <= tolerance, rel
    del interior


@pytest.mark.parametrize("grid_args", GRIDS)
@pytest.mark.parametrize("cnpar", CNPARS)
def test_mixing_from_bottom_and_surface(grid_args, cnpar):
    T = _setup(grid_args)
    nuh = np.full((T.nz + 1, T.ny_, T.nx_), 0.01)
    for level in (0, -1):
        tracer = np.zeros((T.nz, T.ny_, T.nx_))
        tracer[level] = 1.0
        _diffuse(T, tracer, nuh, cnpar)


@pytest.mark.parametrize("grid_args", GRIDS)
@pytest.mark.parametrize("cnpar", CNPARS)
def test_source(grid_args, cnpar):
    T = _setup(grid_args)
    nuh = np.full((T.nz + 1, T.ny_, T.nx_), 0.01)
    tracer = np.zeros((T.nz, T.ny_, T.nx_))
    sources = (1.0 / DT) * DT * T.hn
    _diffuse(T, tracer, nuh, cnpar, sources=np.ascontiguousarray(sources))


@pytest.mark.parametrize("grid_args", GRIDS)
def test_relative_source(grid_args):
    """python/tests/test_vertical_diffusion.py:174-205: linear source only
    gives 1/(1-r)^N to 1e-13."""
    T = _setup(grid_args)
    nuh = np.full((T.nz + 1, T.ny_, T.nx_), 0.01)
    vdif = O.VerticalDiffusion(T, cnpar=1.0)
    tracer = np.ones((T.nz, T.ny_, T.nx_))
    r = 0.1
    rel_sources = np.ascontiguousarray((r / DT) * DT * T.hn)
    for _ in range(NSTEP):
        vdif(nuh, DT, tracer, ea2=rel_sources)
    expected = 1.0 / (1.0 - r) ** NSTEP
    wet = T.mask == 1
    rel = (tracer[:, wet] - expected) / expected
    assert not (rel.min(axis=1) - rel.max(axis=1)).any()
    assert np.abs(rel).max() <= 1e-13


@pytest.mark.parametrize("grid_args", GRIDS)
@pytest.mark.parametrize("cnpar", CNPARS)
@pytest.mark.parametrize("seed", [1, 2])
def test_random_diffusivity_random_tracer_with_sources_changing_h(grid_args, cnpar, seed):
    """python/tests/test_vertical_diffusion.py:255-271"""
    rng = np.random.default_rng(seed)
    T = _setup(grid_args)
    nuh = np.broadcast_to(10.0 ** rng.uniform(-6.0, 0.0, (T.nz + 1, 1, 1)), (T.nz + 1, T.ny_, T.nx_)).copy()
    tracer = np.broadcast_to(rng.uniform(0.0, 1.0, (T.nz, 1, 1)), (T.nz, T.ny_, T.nx_)).copy()
    src = np.broadcast_to(rng.uniform(0.0, 1.0, (T.nz, 1, 1)), (T.nz, T.ny_, T.nx_))
    sources = np.ascontiguousarray(src * DT * T.hn)
    _diffuse(T, tracer, nuh, cnpar, tolerance=1e-11, sources=sources, change_ho=True, rng=rng)


@pytest.mark.parametrize("cnpar", CNPARS)
def test_random_diffusivity(cnpar):
    rng = np.random.default_rng(5)
    T = _setup({})
    nuh = np.broadcast_to(10.0 ** rng.uniform(-6.0, 0.0, (T.nz + 1, 1, 1)), (T.nz + 1, T.ny_, T.nx_)).copy()
    tracer = np.full((T.nz, T.ny_, T.nx_), 35.0)
    _diffuse(T, tracer, nuh, cnpar, tolerance=1e-11)


def test_single_layer_shortcut():
    """diffusion.F90:224-231: nz == 1 gives var = (ho*var + ea4)/(hn - ea2)
    at every point."""
    T = _setup({})
    rng = np.random.default_rng(3)
    T1 = O.make_grids(column_grid(nz=1)[0])
    T1.hn[...] = rng.uniform(1, 2, T1.hn.shape)
    T1.ho[...] = rng.uniform(1, 2, T1.hn.shape)
    var = rng.uniform(0, 1, T1.hn.shape)
    ea2 = rng.uniform(0, 0.1, T1.hn.shape)
    ea4 = rng.uniform(0, 0.1, T1.hn.shape)
    expected = (T1.ho * var + ea4) / (T1.hn - ea2)
    v = O.VerticalDiffusion(T1)
    nuh = np.zeros((2,) + T1.hn.shape[1:])
    v(nuh, DT, var, ea2=ea2, ea4=ea4, use_ho=True)
    assert np.array_equal(var, expected)
    del T


@pytest.mark.parametrize("cnpar", [0.5, 1.0])
def test_gaussian_against_the_analytic_solution(cnpar):
    """tests/test_vertical_diffusion.F90:14-75, 145-160 (initial_conditions
    method 1): a Gaussian of amplitude 5 and width 5 m in a 100 m column of
    100 one-metre layers, constant diffusivity 0.1 m2/s, 200 steps of 5 s.
    The analytic solution stays Gaussian, amplitude 5 sqrt(a^2/C),
    C = 4 Av t + a^2.  The discretisation error is 7e-4 of the amplitude
    (both weights); the column total is conserved to rounding."""
    wet, var, ana, total0, total = gaussian_column(O.VerticalDiffusion, cnpar)
    assert np.abs(var[:, wet] - ana[:, None]).max() / GAUSS["cmax"] < 1.5e-3
    assert np.abs(total - total0).max() / total0.max() < 1e-13


GAUSS = dict(nz=100, depth=100.0, Av=0.1, cmax=5.0, a=5.0, dt=5.0, nstep=200)


def gaussian_column(make_diffusion, cnpar, to_device=None, from_device=None, nx=6, ny=5):
    """The column of tests/test_vertical_diffusion.F90 on an nx x ny patch of
    identical columns, diffused by ``make_diffusion(grid, cnpar)`` (the
    oracle's, or a device one with ``to_device``/``from_device`` moving the
    grid and fields); returns (wet mask, final field, analytic profile,
    column totals before and after)."""
    g = GAUSS
    nz, depth = g["nz"], g["depth"]
    Th, dga, hn = column_grid(nx=nx, ny=ny, nz=nz, H=depth, land=0.0)
    dz = depth / nz
    z = -depth + dz * np.arange(nz)  # level positions of the F90 program (z(1) = -depth)
    z0 = z[nz // 2 - 1]
    var = np.broadcast_to((g["cmax"] * np.exp(-(z - z0) ** 2 / g["a"] ** 2))[:, None, None], hn.shape).copy()
    nuh = np.full((nz + 1,) + hn.shape[1:], g["Av"])
    if to_device is None:
        T = O.make_grids(Th)
        T.hn[...] = hn
        T.ho[...] = hn
        wet = T.mask == 1
        total0 = (var * hn)[:, wet].sum(axis=0)
        vd = make_diffusion(T, cnpar)
        for _ in range(g["nstep"]):
            vd(nuh, g["dt"], var)
    else:
        wet = Th.mask == 1
        total0 = (var * hn)[:, wet].sum(axis=0)
        var = from_device(to_device(make_diffusion, Th, hn, nuh, var, cnpar, g["dt"], g["nstep"]))
    C1 = 4.0 * g["Av"] * g["nstep"] * g["dt"] + g["a"] ** 2
    ana = g["cmax"] * np.sqrt(g["a"] ** 2 / C1) * np.exp(-(z - z0) ** 2 / C1)
    total = (var * hn)[:, wet].sum(axis=0)
    return wet, var, ana, total0, total
