"""Parity of the CUDA operators (called through the C ABI via the pygetm-style
API) with the CPU oracle on identical seeded inputs.

Tolerance: FP64, 1e-12 relative to the field's magnitude per kernel call and
1e-11 for a full 5-pass Strang split (the GPU contracts multiply-adds into
FMAs, the oracle does not; most points agree bit for bit, and HSIMT's
1/(1-cfl) term amplifies the last-bit differences of the rest)."""

import numpy as np
import pytest

from tests.gpu_helpers import apply_state_device, apply_state_oracle, dev, host, random_state
from tests.helpers import full_grid

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def close(a, b, rtol=RTOL, mask=None):
    a = np.asarray(a)
    b = np.asarray(b)
    if mask is not None:
        a = a[..., mask]
        b = b[..., mask]
    fin = np.isfinite(b)
    assert np.array_equal(fin, np.isfinite(a)), "non-finite pattern differs"
    scale = max(np.abs(b[fin & (np.abs(b) < 1e15)]).max(initial=0.0), 1e-300)
    err = np.abs(a[fin] - b[fin])
    big = np.abs(b[fin]) >= 1e15  # FILL_VALUE-scaled garbage in masked points
    err = np.where(big, err / np.abs(b[fin]).clip(1.0), err / scale)
    assert err.max(initial=0.0) <= rtol, f"max relative error {err.max()}"
    return err.max(initial=0.0)


def setup(nz=8, seed=0, f=0.0, nx=40, ny=30):
    import oracle.oracle as O
    from getm_gb300.core import make_grids

    Th, rng = full_grid(nx=nx, ny=ny, nz=nz, seed=seed, f=f)
    state = random_state(Th, rng, nz)
    To = O.make_grids(Th)
    apply_state_oracle(To, state)
    Td = make_grids(Th)
    apply_state_device(Td, state)
    return Th, To, Td, rng


def wrap(grid, a, z):
    from getm_gb300.core import Array

    return Array(grid, dev(a), z=z)


def velocity(g, rng, nz, scale):
    v = rng.uniform(-scale, scale, (nz, g.ny_, g.nx_))
    v[:, g.mask == 0] = 0.0
    return v


@pytest.mark.parametrize("scheme", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("ufirst", [False, True])
def test_apply_3d_batch(scheme, ufirst):
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=scheme)
    nz = Th.nz
    # moderate Courant numbers and tracers bounded away from 0, so no cell is
    # drained (h f - dt advn would then cancel and inflate relative errors)
    u = velocity(Th.ugrid, rng, nz, 0.3)
    v = velocity(Th.vgrid, rng, nz, 0.3)
    w = rng.uniform(-5e-4, 5e-4, (nz + 1, Th.ny_, Th.nx_))
    w[0] = 0.0
    w[-1] = 0.0
    tr = [rng.uniform(5.0, 10.0, (nz, Th.ny_, Th.nx_)) for _ in range(3)]
    Ah_u = rng.uniform(0, 50.0, (Th.ny_, Th.nx_)) if scheme % 2 else None
    Ah_v = rng.uniform(0, 50.0, (Th.ny_, Th.nx_)) if scheme % 2 else None
    dt = 600.0
    ao = O.Advection(To, scheme)
    ao.ufirst = ufirst
    tro = [t.copy() for t in tr]
    ao.apply_3d_batch(u, v, w, dt, tro, Ah_u=Ah_u, Ah_v=Ah_v)
    ad = operators.Advection(Td, operators.AdvectionScheme(scheme))
    ad.ufirst = ufirst
    trd = [wrap(Td, t, CENTERS) for t in tr]
    ad.apply_3d_batch(wrap(Td.ugrid, u, CENTERS), wrap(Td.vgrid, v, CENTERS), wrap(Td, w, INTERFACES), dt, trd,
                      Ah_u=None if Ah_u is None else wrap(Td.ugrid, Ah_u, False),
                      Ah_v=None if Ah_v is None else wrap(Td.vgrid, Ah_v, False))
    for a, b in zip(trd, tro):
        close(host(a.all_values), b, rtol=1e-11)
    close(host(ad.h), ao.h)


def test_vertical_substeps_and_restart():
    """Columns with vertical Courant numbers above 1 take several sub-steps
    (advection.F90.template:286-368)."""
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=11)
    nz = Th.nz
    # Courant numbers up to ~4 from w_var; w moves thicknesses by up to ~20 %
    # so some columns need more sub-steps after the first and restart
    w = rng.uniform(-5e-4, 5e-4, (nz + 1, Th.ny_, Th.nx_))
    w_var = rng.uniform(-0.02, 0.02, (nz + 1, Th.ny_, Th.nx_))
    for a in (w, w_var):
        a[0] = 0.0
        a[-1] = 0.0
    t = rng.uniform(0.0, 1.0, (nz, Th.ny_, Th.nx_))
    for scheme in (1, 5):
        ao = O.VerticalAdvection(To, scheme)
        to = t.copy()
        ao(w, w_var, 600.0, to)
        ad = operators.VerticalAdvection(Td, operators.AdvectionScheme(scheme))
        td = wrap(Td, t, CENTERS)
        ad(wrap(Td, w, INTERFACES), wrap(Td, w_var, INTERFACES), 600.0, td)
        close(host(td.all_values), to)
        close(host(ad.h), ao.h)
    assert O._lib  # oracle loaded


@pytest.mark.parametrize("direction", [1, 2])
def test_single_passes(direction):
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS

    Th, To, Td, rng = setup(seed=20 + direction)
    nz = Th.nz
    g = Th.ugrid if direction == 1 else Th.vgrid
    vel = velocity(g, rng, nz, 1.0)
    t = rng.uniform(0.0, 1.0, (nz, Th.ny_, Th.nx_))
    ao = O.Advection(To, 5)
    ao.h[...] = To.ho
    to = t.copy()
    ad = operators.Advection(Td, operators.AdvectionScheme.SUPERBEE)
    ad.h.copy_(Td.ho.all_values)
    td = wrap(Td, t, CENTERS)
    gd = Td.ugrid if direction == 1 else Td.vgrid
    if direction == 1:
        ao.u_3d(vel, 300.0, to)
        ad.u_3d(wrap(gd, vel, CENTERS), 300.0, td)
    else:
        ao.v_3d(vel, 300.0, to)
        ad.v_3d(wrap(gd, vel, CENTERS), 300.0, td)
    close(host(td.all_values), to)
    close(host(ad.h), ao.h)


@pytest.mark.parametrize("split", [1, 2, 3])
@pytest.mark.parametrize("ufirst", [False, True])
def test_advection_2d_split(split, ufirst):
    import oracle.oracle as O
    from getm_gb300 import operators

    Th, To, Td, rng = setup(seed=30 + split)
    u = velocity(Th.ugrid, rng, 1, 0.5)[0]
    v = velocity(Th.vgrid, rng, 1, 0.5)[0]
    t = rng.uniform(0.0, 1.0, (Th.ny_, Th.nx_))
    ao = O.Advection(To, 5, O.AdvectionSplit(split))
    ao.ufirst = ufirst
    to = t.copy()
    ao(u, v, 600.0, to)
    ad = operators.Advection(Td, operators.AdvectionScheme.SUPERBEE, operators.AdvectionSplit(split))
    ad.ufirst = ufirst
    td = wrap(Td, t, False)
    ad(wrap(Td.ugrid, u, False), wrap(Td.vgrid, v, False), 600.0, td)
    close(host(td.all_values), to)
    close(host(ad.D), ao.D)


@pytest.mark.parametrize("cnpar", [0.5, 1.0])
@pytest.mark.parametrize("use_ho", [False, True])
def test_vertical_diffusion(cnpar, use_ho):
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=40, nz=12)
    nz = Th.nz
    nuh = 10.0 ** rng.uniform(-6, -1, (nz + 1, Th.ny_, Th.nx_))
    t = rng.uniform(0, 1, (nz, Th.ny_, Th.nx_))
    ea2 = rng.uniform(0, 0.1, t.shape)
    ea4 = rng.uniform(0, 0.1, t.shape)
    vo = O.VerticalDiffusion(To, cnpar)
    to = t.copy()
    vo(nuh, 600.0, to, molecular=1e-6, ea2=ea2, ea4=ea4, use_ho=use_ho)
    vd = operators.VerticalDiffusion(Td, cnpar)
    # fused path
    td = wrap(Td, t, CENTERS)
    vd(wrap(Td, nuh, INTERFACES), 600.0, td, molecular=1e-6, ea2=wrap(Td, ea2, CENTERS), ea4=wrap(Td, ea4, CENTERS), use_ho=use_ho)
    close(host(td.all_values), to)
    # prepare + apply path
    td2 = wrap(Td, t, CENTERS)
    vd.prepare(wrap(Td, nuh, INTERFACES), 600.0, 1e-6, use_ho)
    vd.apply(td2, wrap(Td, ea2, CENTERS), wrap(Td, ea4, CENTERS), use_ho)
    close(host(td2.all_values), to)


def test_tracer_transport_steps():
    """Several steps of the tracer-transport configuration (advection of the
    tracer blob + vertical diffusion) on a reduced grid."""
    from getm_gb300 import workloads
    from getm_gb300.simulation import TracerTransport as GT
    from oracle.models import TracerTransport as OT

    wl = workloads.tracer_transport(nx=60, ny=50, nz=12)
    g = GT(wl, ntracer=2)
    o = OT(wl, ntracer=2)
    for _ in range(10):
        g.step()
        o.step()
    wet = wl.T.mask == 1
    for a, b in zip(g.tracers._tracers, o.tracers):
        close(host(a.all_values), b, rtol=1e-11, mask=wet)
