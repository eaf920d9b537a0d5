"""Per-call parity of the momentum-side kernels with the oracle on identical
seeded inputs: momentum_diffusion (2D and 3D), horizontal_diffusion,
shear_frequency, shear_frequency2, surface_shear_velocity,
bottom_shear_velocity, thickness2center_depth, the Coriolis terms (DEFAULT
and ESPELID, 2D and 3D), vertical_advection_to_sources and update_gvc.
These are the _pygetm calls of python/_pygetm.pyx:318-585 behind
python/src/wrapper.F90:275-600 and python/src/momentum.F90:12-321, and
python/pygetm/momentum.py:1127-1148.

Tolerance: FP64, 1e-12 relative to the field's magnitude (the GPU contracts
multiply-adds, the oracle does not)."""

import numpy as np
import pytest

from tests.gpu_helpers import dev, host
from tests.test_gpu_operators import close, setup, velocity, wrap

pytestmark = pytest.mark.gpu


def _report(name, err):
    print(f"{name}: max relative error {err:.3e}")


@pytest.mark.parametrize("three_d", [False, True])
def test_momentum_diffusion(three_d):
    """wrapper.F90:275-393: diffusion of u and v with Am0 on the UU/UV/VU/VV
    thicknesses (2D: the depth-averaged velocities and depths; 3D: every
    layer with the layer thicknesses)."""
    import oracle.oracle as O
    from getm_gb300 import _pygetm
    from getm_gb300.core import CENTERS

    Th, To, Td, rng = setup(seed=50 + three_d, nz=6)
    ug, vg = Th.ugrid, Th.vgrid
    nz = Th.nz
    if three_d:
        u = velocity(ug, rng, nz, 0.8)
        v = velocity(vg, rng, nz, 0.8)
        hs = [To.ugrid.ugrid.hn, To.ugrid.vgrid.hn, To.vgrid.ugrid.hn, To.vgrid.vgrid.hn]
        z = CENTERS
    else:
        u = velocity(ug, rng, 1, 0.8)[0]
        v = velocity(vg, rng, 1, 0.8)[0]
        hs = [To.ugrid.ugrid.D, To.ugrid.vgrid.D, To.vgrid.ugrid.D, To.vgrid.vgrid.D]
        z = False
    Am = 55.0
    du0 = rng.uniform(-1, 1, u.shape)
    dv0 = rng.uniform(-1, 1, v.shape)
    du_o, dv_o = du0.copy(), dv0.copy()
    O.momentum_diffusion(To.ugrid, To.vgrid, *[np.ascontiguousarray(h) for h in hs], u, v, Am, du_o, dv_o)
    Ud, Vd = Td.ugrid, Td.vgrid
    src = [Ud.ugrid, Ud.vgrid, Vd.ugrid, Vd.vgrid]
    hd = [g.hn if three_d else g.D for g in src]
    du, dv = wrap(Ud, du0, z), wrap(Vd, dv0, z)
    _pygetm.momentum_diffusion(*hd, wrap(Ud, u, z), wrap(Vd, v, z), Am, du, dv)
    assert np.abs(du_o - du0).max() > 0.0  # the call did write
    _report("diffu", close(host(du.all_values), du_o))
    _report("diffv", close(host(dv.all_values), dv_o))


@pytest.mark.parametrize("on", ["T", "U"])
def test_horizontal_diffusion(on):
    """pyx:369-390 (momentum.F90:12-77): the numerical damping of a 2D field
    with diffusivities on the field grid's U and V grids; on the U grid as
    Momentum.update_depth_integrated_diagnostics uses it for dampU."""
    import oracle.oracle as O
    from getm_gb300 import _pygetm

    Th, To, Td, rng = setup(seed=60)
    go = To if on == "T" else To.ugrid
    gd = Td if on == "T" else Td.ugrid
    gh = Th if on == "T" else Th.ugrid
    f = rng.uniform(-2.0, 2.0, (gh.ny_, gh.nx_))
    f[gh.mask == 0] = 0.0
    Ah_u = rng.uniform(0.0, 80.0, (gh.ny_, gh.nx_))
    Ah_v = rng.uniform(0.0, 80.0, (gh.ny_, gh.nx_))
    out0 = rng.uniform(-1, 1, f.shape)
    out_o = out0.copy()
    O.horizontal_diffusion(go, f, Ah_u, Ah_v, 30.0, out_o)
    out_d = wrap(gd, out0, False)
    _pygetm.horizontal_diffusion(wrap(gd, f, False), wrap(gd.ugrid, Ah_u, False), wrap(gd.vgrid, Ah_v, False), 30.0,
                                 out_d)
    assert np.abs(out_o - out0).max() > 0.0
    _report(f"horizontal_diffusion on {on}", close(host(out_d.all_values), out_o))


def test_shear_frequency():
    """momentum.F90:218-241: squared shear frequency at the interior
    interfaces from uk, vk and the U/V layer thicknesses."""
    import oracle.oracle as O
    from getm_gb300 import _pygetm
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=61, nz=10)
    nz = Th.nz
    uk = velocity(Th.ugrid, rng, nz, 0.5)
    vk = velocity(Th.vgrid, rng, nz, 0.5)
    SS0 = rng.uniform(0, 1e-3, (nz + 1, Th.ny_, Th.nx_))
    SS_o = SS0.copy()
    O.shear_frequency(To, uk, vk, SS_o)
    SS_d = wrap(Td, SS0, INTERFACES)
    _pygetm.shear_frequency(wrap(Td.ugrid, uk, CENTERS), wrap(Td.vgrid, vk, CENTERS), SS_d)
    assert np.abs(SS_o - SS0).max() > 0.0
    _report("SS", close(host(SS_d.all_values), SS_o))


def test_surface_and_bottom_shear_velocity():
    """momentum.F90:270-321: ustar at the surface from the wind stress, and
    at the bottom from the bottom velocities and drag (with the stresses
    ustar2_x, ustar2_y on the U and V grids)."""
    import oracle.oracle as O
    from getm_gb300 import _pygetm

    Th, To, Td, rng = setup(seed=62)
    taux = rng.uniform(-0.3, 0.3, (Th.ny_, Th.nx_))
    tauy = rng.uniform(-0.3, 0.3, (Th.ny_, Th.nx_))
    us0 = rng.uniform(0, 1, taux.shape)
    us_o = us0.copy()
    O.surface_shear_velocity(To, taux, tauy, us_o)
    us_d = wrap(Td, us0, False)
    _pygetm.surface_shear_velocity(wrap(Td, taux, False), wrap(Td, tauy, False), us_d)
    assert np.abs(us_o - us0).max() > 0.0
    _report("ustar_s", close(host(us_d.all_values), us_o))

    ub = velocity(Th.ugrid, rng, 1, 0.6)[0]
    vb = velocity(Th.vgrid, rng, 1, 0.6)[0]
    rru = rng.uniform(1e-4, 5e-3, ub.shape)
    rrv = rng.uniform(1e-4, 5e-3, vb.shape)
    outs0 = [rng.uniform(0, 1, ub.shape), rng.uniform(0, 1, vb.shape), rng.uniform(0, 1, taux.shape)]
    outs_o = [x.copy() for x in outs0]
    O.bottom_shear_velocity(To, ub, vb, rru, rrv, *outs_o)
    grids = [Td.ugrid, Td.vgrid, Td]
    outs_d = [wrap(g, x, False) for g, x in zip(grids, outs0)]
    _pygetm.bottom_shear_velocity(wrap(Td.ugrid, ub, False), wrap(Td.vgrid, vb, False), wrap(Td.ugrid, rru, False),
                                  wrap(Td.vgrid, rrv, False), *outs_d)
    for name, a, b, x0 in zip(("ustar2_x", "ustar2_y", "ustar_b"), outs_d, outs_o, outs0):
        assert np.abs(b - x0).max() > 0.0
        _report(name, close(host(a.all_values), b))


def test_thickness2center_depth():
    """wrapper.F90:395-407: depth of each layer centre below the surface."""
    import oracle.oracle as O
    from getm_gb300 import _pygetm
    from getm_gb300.core import CENTERS

    Th, To, Td, rng = setup(seed=63, nz=12)
    out_o = np.zeros((Th.nz, Th.ny_, Th.nx_))
    O.thickness2center_depth(To, To.hn, out_o)
    out_d = wrap(Td, np.zeros_like(out_o), CENTERS)
    _pygetm.thickness2center_depth(Td.mask, Td.hn, out_d)
    _report("center depth", close(host(out_d.all_values), out_o))


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("three_d", [False, True])
def test_coriolis(scheme, three_d):
    """momentum.py:1127-1148: the Coriolis term of U on the V grid (negated)
    and of V on the U grid, DEFAULT (plain interpolation) and ESPELID
    (sqrt-depth weighted) schemes; compared on water points of the target
    (the reference leaves ESPELID's land points unset)."""
    from getm_gb300.core import CENTERS
    from getm_gb300.momentum import CoriolisScheme, Momentum
    from oracle.models import Momentum as OMomentum

    Th, To, Td, rng = setup(seed=64 + scheme, nz=5, f=1.2e-4)
    nz = Th.nz
    om = OMomentum(coriolis_scheme=scheme)
    gm = Momentum(coriolis_scheme=CoriolisScheme(scheme))
    gm.fused_2d = True
    z = CENTERS if three_d else False
    for src_h, dst_h, src_o, dst_o, src_d, dst_d, xdir in (
            (Th.ugrid, Th.vgrid, To.ugrid, To.vgrid, Td.ugrid, Td.vgrid, True),
            (Th.vgrid, Th.ugrid, To.vgrid, To.ugrid, Td.vgrid, Td.ugrid, False)):
        U = velocity(src_h, rng, nz, 2.0) * (10.0 if not three_d else 1.0)
        if not three_d:
            U = U[0]
        out0 = rng.uniform(-1e-3, 1e-3, (nz, dst_h.ny_, dst_h.nx_) if three_d else (dst_h.ny_, dst_h.nx_))
        out_o = out0.copy()
        om.coriolis(src_o, U, dst_o, out_o, xdir)
        out_d = wrap(dst_d, out0, z)
        gm.coriolis(wrap(src_d, U, z), out_d, xdir)
        wet = dst_h.mask != 0
        _report(f"coriolis scheme {scheme} {'3D' if three_d else '2D'} x={xdir}",
                close(host(out_d.all_values), out_o, mask=wet))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_shear_frequency2(dtype):
    """momentum.F90:244-268: the viscosity-weighted squared shear frequency
    (pyx:468-479); FP64 to 1e-12 of the field's magnitude, float uk, vk,
    num, SS to 1e-5."""
    import torch

    import oracle.oracle as O
    from getm_gb300 import _pygetm
    from getm_gb300.core import CENTERS, INTERFACES, Array

    Th, To, Td, rng = setup(seed=64, nz=10)
    nz = Th.nz
    uk = velocity(Th.ugrid, rng, nz, 0.5)
    vk = velocity(Th.vgrid, rng, nz, 0.5)
    num = rng.uniform(1e-5, 1e-2, (nz + 1, Th.ny_, Th.nx_))
    if dtype == "float32":
        uk, vk, num = (x.astype(np.float32).astype(np.float64) for x in (uk, vk, num))
    SS0 = rng.uniform(0, 1e-3, (nz + 1, Th.ny_, Th.nx_))
    SS_o = SS0.copy()
    O.shear_frequency2(To, uk, vk, num, SS_o)
    td = torch.float64 if dtype == "float64" else torch.float32
    wrapt = lambda g, a, z: Array(g, dev(a).to(td), z=z)  # noqa: E731
    SS_d = wrapt(Td, SS0, INTERFACES)
    _pygetm.shear_frequency2(wrapt(Td.ugrid, uk, CENTERS), wrapt(Td.vgrid, vk, CENTERS), wrapt(Td, num, INTERFACES),
                             SS_d)
    assert np.abs(SS_o - SS0).max() > 0.0
    _report("SS2 " + dtype, close(host(SS_d.all_values).astype(np.float64), SS_o,
                                  1e-12 if dtype == "float64" else 1e-5))


def test_vertical_advection_to_sources():
    """wrapper.F90:447-485 (pyx:574-575): upstream vertical fluxes of a
    sinking or floating field into its source term, against the oracle; and
    no change at all when w is zero at every interior point."""
    import torch

    import oracle.oracle as O
    from getm_gb300 import _pygetm

    rng = np.random.default_rng(65)
    nz, ny, nx = 12, 30, 41
    mask = (rng.uniform(size=(nz, ny, nx)) > 0.1).astype(np.int32)
    c = rng.uniform(0.5, 2.0, (nz, ny, nx))
    h = rng.uniform(1.0, 3.0, (nz, ny, nx))
    w = rng.uniform(-1e-3, 1e-3, (nz, ny, nx))
    s0 = rng.uniform(-1e-6, 1e-6, (nz, ny, nx))
    s_o = s0.copy()
    O.vertical_advection_to_sources(2, 3, mask, c, w, h, s_o)
    s_d = dev(s0)
    _pygetm.vertical_advection_to_sources(2, 3, dev(mask), dev(c), dev(w), dev(h), s_d)
    _report("vadv sources", close(host(s_d), s_o, 1e-14))
    # w zero in the interior (non-zero in the halos), NaN in c: unchanged
    w2 = np.zeros_like(w)
    w2[:, :3] = 1.0
    c[3, 10, 10] = np.nan
    s_d = dev(s0)
    _pygetm.vertical_advection_to_sources(2, 3, dev(mask), dev(c), dev(w2), dev(h), s_d)
    torch.cuda.synchronize()
    assert np.array_equal(host(s_d), s0)


def test_update_gvc():
    """wrapper.F90:567-600 (pyx:577-585): general vertical coordinates
    against the oracle (1e-14: the GPU contracts the blend into a fused
    multiply-add)."""
    import torch

    import oracle.oracle as O
    from getm_gb300 import _pygetm
    from getm_gb300.domain import calculate_sigma

    rng = np.random.default_rng(66)
    nz, ny, nx = 20, 33, 47
    dbeta = calculate_sigma(nz, 2.0, 1.0)
    D = rng.uniform(2.0, 400.0, (ny, nx))
    mask = (rng.uniform(size=(ny, nx)) > 0.2).astype(np.int32)
    h0 = rng.uniform(size=(nz, ny, nx))
    for kk in (-1, 0):
        h_o = h0.copy()
        O.update_gvc(1.0 / nz, dbeta, 30.0, kk, D, mask, h_o)
        h_d = dev(h0)
        _pygetm.update_gvc(1.0 / nz, dev(dbeta), 30.0, kk, dev(D), dev(mask), h_d)
        torch.cuda.synchronize()
        _report(f"gvc kk={kk}", close(host(h_d), h_o, 1e-14))
