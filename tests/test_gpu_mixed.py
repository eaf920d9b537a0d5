"""The mixed-precision form against the FP64 oracle / FP64 GPU path.

Fluxes, limiters and tridiagonal solves run in float32 (in increment form:
the change of a field is formed from differences of neighbouring values);
elevations, depths, layer thicknesses, density and the internal pressure
gradient stay float64.
Tolerances are stated per test: a few float32 ulps (about 1e-6 relative) per
operator call, 1e-5 relative for tracers after several full split-explicit
steps, and an absolute bound for the elevation of an unforced box."""

import numpy as np
import pytest

from tests.gpu_helpers import dev, host
from tests.test_gpu_operators import setup, velocity

pytestmark = pytest.mark.gpu


def rel(a, b, mask=None):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    if mask is not None:
        a, b = a[..., mask], b[..., mask]
    return float(np.abs(a - b).max() / np.abs(b).max())


def wrap32(grid, a, z):
    from getm_gb300.core import Array

    return Array(grid, dev(a).float(), z=z)


@pytest.mark.parametrize("scheme", [1, 5, 6])
def test_apply_3d_batch_f32(scheme):
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=50 + scheme)
    nz = Th.nz
    u = velocity(Th.ugrid, rng, nz, 0.3)
    v = velocity(Th.vgrid, rng, nz, 0.3)
    w = rng.uniform(-5e-4, 5e-4, (nz + 1, Th.ny_, Th.nx_))
    w[0] = w[-1] = 0.0
    # inputs rounded to float32 so both sides start from identical values
    u, v, w = (x.astype(np.float32).astype(np.float64) for x in (u, v, w))
    tr = [rng.uniform(5.0, 10.0, (nz, Th.ny_, Th.nx_)).astype(np.float32).astype(np.float64) for _ in range(2)]
    ao = O.Advection(To, scheme)
    tro = [t.copy() for t in tr]
    ao.apply_3d_batch(u, v, w, 600.0, tro)
    ad = operators.Advection(Td, operators.AdvectionScheme(scheme))
    trd = [wrap32(Td, t, CENTERS) for t in tr]
    ad.apply_3d_batch(wrap32(Td.ugrid, u, CENTERS), wrap32(Td.vgrid, v, CENTERS), wrap32(Td, w, INTERFACES), 600.0, trd)
    wet = Th.mask == 1
    # HSIMT's 1/(1-cfl) term amplifies float32 rounding
    tol = 1e-5 if scheme == 1 else 5e-6
    for a, b in zip(trd, tro):
        assert rel(host(a.all_values), b, wet) < tol
    # layer thicknesses are stored and updated in float64; in the mixed form
    # the transports that change them are evaluated in float32
    assert rel(host(ad.h), ao.h, wet) < 1e-6


def test_vertical_diffusion_f32():
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=60, nz=12)
    nz = Th.nz
    nuh = (10.0 ** rng.uniform(-6, -1, (nz + 1, Th.ny_, Th.nx_))).astype(np.float32).astype(np.float64)
    t = rng.uniform(0, 1, (nz, Th.ny_, Th.nx_)).astype(np.float32).astype(np.float64)
    vo = O.VerticalDiffusion(To, 1.0)
    to = t.copy()
    vo(nuh, 600.0, to, molecular=1e-6)
    vd = operators.VerticalDiffusion(Td, 1.0)
    td = wrap32(Td, t, CENTERS)
    vd(wrap32(Td, nuh, INTERFACES), 600.0, td, molecular=1e-6)
    assert rel(host(td.all_values), to, Th.mask == 1) < 2e-6


@pytest.mark.parametrize("scheme", [1, 5, 6])
def test_apply_3d_batch_f64s(scheme):
    """FP64-stored tracers with float velocities and float increments
    (getm_advection_apply_3d_batch_f64s): fields of a large mean plus a small
    signal, where float32 storage could not even hold the change; the change
    matches the FP64 oracle to float32 accuracy (1e-5 of its largest value;
    HSIMT 2e-5), the thicknesses to 1e-6."""
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import Array, CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=80 + scheme)
    nz = Th.nz
    u = velocity(Th.ugrid, rng, nz, 0.3)
    v = velocity(Th.vgrid, rng, nz, 0.3)
    w = rng.uniform(-5e-4, 5e-4, (nz + 1, Th.ny_, Th.nx_))
    w[0] = w[-1] = 0.0
    u, v, w = (x.astype(np.float32).astype(np.float64) for x in (u, v, w))
    tr = [1000.0 + rng.uniform(0.0, 1.0, (nz, Th.ny_, Th.nx_)) for _ in range(3)]
    ao = O.Advection(To, scheme)
    tro = [t.copy() for t in tr]
    ao.apply_3d_batch(u, v, w, 600.0, tro)
    ad = operators.Advection(Td, operators.AdvectionScheme(scheme))
    trd = [Array(Td, dev(t), z=CENTERS) for t in tr]
    ad.apply_3d_batch(wrap32(Td.ugrid, u, CENTERS), wrap32(Td.vgrid, v, CENTERS), wrap32(Td, w, INTERFACES), 600.0, trd)
    wet = Th.mask == 1
    tol = 2e-5 if scheme == 1 else 1e-5
    for a, b, t0 in zip(trd, tro, tr):
        assert a.all_values.dtype == __import__("torch").float64
        assert rel(host(a.all_values) - t0, b - t0, wet) < tol
    assert rel(host(ad.h), ao.h, wet) < 1e-6


@pytest.mark.parametrize("sources", [False, True])
def test_vertical_diffusion_f64s(sources):
    """FP64-stored fields diffused with a float solve (getm_vertical_diffusion_
    batch_f64s): the change matches the FP64 oracle to 5e-6 of its largest
    value, for a field of a large mean plus a small signal (diffusivities up
    to 0.1 m2/s over 600 s couple the column strongly; the float Thomas
    sweep's rounding, relative to the change, is a few float32 ulps times
    that conditioning)."""
    import oracle.oracle as O
    from getm_gb300 import operators
    from getm_gb300.core import Array, CENTERS, INTERFACES

    Th, To, Td, rng = setup(seed=90 + sources, nz=12)
    nz = Th.nz
    nuh = (10.0 ** rng.uniform(-6, -1, (nz + 1, Th.ny_, Th.nx_))).astype(np.float32).astype(np.float64)
    t = 500.0 + rng.uniform(0, 1, (nz, Th.ny_, Th.nx_))
    ea4 = rng.uniform(0, 1e-3, t.shape).astype(np.float32).astype(np.float64) if sources else None
    vo = O.VerticalDiffusion(To, 1.0)
    to = t.copy()
    vo(nuh, 600.0, to, molecular=1e-6, ea4=ea4)
    vd = operators.VerticalDiffusion(Td, 1.0)
    td = Array(Td, dev(t), z=CENTERS)
    vd(wrap32(Td, nuh, INTERFACES), 600.0, td, molecular=1e-6, ea4=None if ea4 is None else wrap32(Td, ea4, CENTERS))
    wet = Th.mask == 1
    assert rel(host(td.all_values) - t, to - t, wet) < 5e-6


def test_mixed_seamount_1000_steps():
    """The full 400 x 300 x 40 seamount for 1000 3D steps in the mixed form
    (FP64 tracer storage, float increments, velocities and solves) against
    the FP64 form: temperature within 1e-5 of its largest value, salinity
    within 1e-10.  (The elevation of this unforced box is a residual signal
    of 2e-6 m; its error is reported, not bounded relative to that signal:
    FP64 itself, restarted from a temperature moved by one ulp, differs by
    1e-4 of it after 1000 steps.)"""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount()
    p = wl.params
    sims = {}
    for prec in ("fp64", "mixed"):
        s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=prec)
        zc = s.T.zc.all_values
        temp0 = torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                            s.temp.all_values.double()).float().double()
        s.temp.all_values.copy_(temp0)
        s.start(p["timestep"], p["split_factor"])
        sims[prec] = s
    n = 1000 * p["split_factor"]
    for prec, s in sims.items():
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        graphs = []
        with torch.cuda.stream(stream):
            for _ in range(2 * p["split_factor"]):  # warm-up: allocate work buffers
                s.advance()
            for _ in range(2):  # one graph per parity of the 3D step (captures run nothing)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=stream):
                    for _ in range(p["split_factor"]):
                        s.advance()
                graphs.append(g)
        torch.cuda.current_stream().wait_stream(stream)
        done = 2 * p["split_factor"]  # substeps run by the warm-up
        while done < n:
            graphs[(done // p["split_factor"]) % 2].replay()
            done += p["split_factor"]
        torch.cuda.synchronize()
        assert s.split2d_status() == 0
    a, b = sims["mixed"], sims["fp64"]
    assert a.temp.all_values.dtype == torch.float64
    wet = wl.T.mask == 1
    e = {"temp": rel(host(a.temp.all_values), host(b.temp.all_values), wet),
         "salt": rel(host(a.salt.all_values), host(b.salt.all_values), wet),
         "z_abs_m": float(np.abs(host(a.T.z.all_values) - host(b.T.z.all_values))[wet].max())}
    print("mixed vs fp64 after 1000 3D steps:", {k: f"{v:.2e}" for k, v in e.items()})
    assert e["temp"] < 1e-5
    assert e["salt"] < 1e-10


def test_mixed_simulation_error_vs_fp64():
    """Several 3D steps of the seamount box in both forms from identical
    (float32-representable) initial fields.  Tracer errors of the mixed form
    relative to FP64 stay below 1e-5.  The elevation of this unforced box is
    a tiny signal, so its error is compared with the effect of rounding the
    initial temperature to float32 in a pure FP64 run (the conditioning of
    the problem itself)."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount(nx=40, ny=30, nz=10, dx=10000.0)
    p = wl.params
    sims = {}
    for key, prec, rounded in (("fp64", "fp64", True), ("fp64_raw", "fp64", False), ("mixed", "mixed", True)):
        s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=prec)
        zc = s.T.zc.all_values
        temp0 = torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0, s.temp.all_values.double())
        if rounded:
            temp0 = temp0.float().double()
        s.temp.all_values.copy_(temp0)
        s.start(10.0, 10)
        for _ in range(50):
            s.advance()
        sims[key] = s
    wet = wl.T.mask == 1

    def errs(a, b):
        z_a, z_b = host(a.T.z.all_values), host(b.T.z.all_values)
        return {"temp": rel(host(a.temp.all_values), host(b.temp.all_values), wet),
                "salt": rel(host(a.salt.all_values), host(b.salt.all_values), wet),
                "z": float(np.abs(z_a - z_b)[wet].max() / np.abs(z_b[wet]).max()),
                "z_abs": float(np.abs(z_a - z_b)[wet].max()), "z_max": float(np.abs(z_b[wet]).max()),
                "U": rel(host(a.momentum.U.all_values), host(b.momentum.U.all_values), wl.T.ugrid.mask == 1),
                "uk": rel(host(a.momentum.uk.all_values), host(b.momentum.uk.all_values), wl.T.ugrid.mask == 1)}

    e_mixed = errs(sims["mixed"], sims["fp64"])
    e_cond = errs(sims["fp64_raw"], sims["fp64"])
    print("mixed vs fp64 after 5 3D steps:", {k: f"{v:.2e}" for k, v in e_mixed.items()})
    print("fp64, initial temperature rounded to float32 vs not:", {k: f"{v:.2e}" for k, v in e_cond.items()})
    assert e_mixed["temp"] < 1e-5
    assert e_mixed["salt"] < 1e-5
    # The unforced box's elevation (under a millimetre) comes from the small
    # residual of the sigma-coordinate pressure gradient, so its relative
    # error is dominated by float32 rounding of the density field (compare
    # e_cond); the absolute elevation error stays below 0.1 mm.
    assert e_mixed["z_abs"] < 1e-4


@pytest.mark.parametrize("split", [1, 2, 3])
def test_advection_2d_mixed(split):
    """2D advection of a float64 field with float32 increments: the change of
    the field matches the FP64 oracle to float32 accuracy (1e-5 of the largest
    change), the column heights to 1e-6."""
    import oracle.oracle as O
    from getm_gb300 import operators
    from tests.test_gpu_operators import wrap

    Th, To, Td, rng = setup(seed=70 + split)
    u = velocity(Th.ugrid, rng, 1, 0.5)[0]
    v = velocity(Th.vgrid, rng, 1, 0.5)[0]
    # a large mean plus a small signal: the increments are what float32 must resolve
    t = 100.0 + rng.uniform(0.0, 1.0, (Th.ny_, Th.nx_))
    ao = O.Advection(To, 5, O.AdvectionSplit(split))
    to = t.copy()
    ao(u, v, 600.0, to)
    ad = operators.Advection(Td, operators.AdvectionScheme.SUPERBEE, operators.AdvectionSplit(split),
                             increments_2d="float32")
    td = wrap(Td, t, False)
    ad(wrap(Td.ugrid, u, False), wrap(Td.vgrid, v, False), 600.0, td)
    wet = Th.mask == 1
    change_gpu = host(td.all_values) - t
    change_ref = to - t
    assert rel(change_gpu, change_ref, wet) < 1e-5
    assert rel(host(ad.D), ao.D, wet) < 1e-6


def test_smcw_mixed_arithmetic():
    """Internal pressure with float slope corrections (mixed form) against
    the FP64 form on a stratified seamount over steep topography, where the
    slope corrections are some 100 times the resulting gradient: 2e-4 of the
    gradient's magnitude (the end-to-end effect on a 1000-step run is below
    that of float32 tracer storage; see the bench's error report)."""
    import torch

    from getm_gb300 import _pygetm, workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount(nx=60, ny=44, nz=12, dx=5000.0)
    p = wl.params
    s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                        s.temp.all_values))
    s.start(10.0, 10)
    s.update_density()
    _pygetm.shchepetkin_mcwilliams(s.buoy, s.idpdx, s.idpdy, arithmetic="float64")
    ref_x, ref_y = s.idpdx.all_values.clone(), s.idpdy.all_values.clone()
    _pygetm.shchepetkin_mcwilliams(s.buoy, s.idpdx, s.idpdy, arithmetic="float32")
    wu = torch.from_numpy(wl.T.ugrid.mask == 1).cuda()
    wv = torch.from_numpy(wl.T.vgrid.mask == 1).cuda()
    ex = float((s.idpdx.all_values - ref_x)[..., wu].abs().max() / ref_x[..., wu].abs().max())
    ey = float((s.idpdy.all_values - ref_y)[..., wv].abs().max() / ref_y[..., wv].abs().max())
    print(f"SMcW float slopes: {ex:.2e} {ey:.2e}")
    assert ex < 2e-4 and ey < 2e-4


def test_density_double_float():
    """Mixed-form density (float S and T, the anomaly rho - rho0 in
    double-float) against the FP64 evaluation of the oracle on the same
    float-valued inputs: the double-float anomaly is the more accurate of the
    two (no cancellation against rho0), so both agree to the FP64 form's own
    rounding of rho (a few ulps of 1026 kg m-3) and of the buoyancy."""
    import torch

    from getm_gb300 import _lib
    from oracle.models import seos_buoyancy

    rng = np.random.default_rng(11)
    n = 200_000
    S = rng.uniform(0.0, 40.0, n).astype(np.float32)
    T = rng.uniform(-2.0, 32.0, n).astype(np.float32)
    z = rng.uniform(0.0, 6000.0, n)
    rho_ref, b_ref = seos_buoyancy(S.astype(np.float64), T.astype(np.float64), z)
    Sd, Td, zd = (torch.from_numpy(a).cuda() for a in (S, T, z))
    rho = torch.empty(n, dtype=torch.float64, device="cuda")
    b = torch.empty_like(rho)
    _lib.call("getm_density_buoyancy_f32", n, Sd.data_ptr(), Td.data_ptr(), zd.data_ptr(), rho.data_ptr(),
              b.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    drho = np.abs(rho.cpu().numpy() - rho_ref).max()
    db = np.abs(b.cpu().numpy() - b_ref).max()
    print(f"double-float density: rho {drho:.2e} kg m-3, buoyancy {db:.2e} m s-2")
    assert drho < 2e-12 and db < 2e-14


def test_density_and_nn_from_fp64_tracers():
    """Mixed form with FP64 tracers: density from FP64 S and T split into
    float pairs (double-float anomaly) against the oracle's FP64 evaluation,
    to FP64 rounding of rho (and 2e-14 m s-2 in buoyancy); the squared
    buoyancy frequency in float arithmetic (differences in FP64) against the
    FP64 kernel to 1e-5 of its largest value."""
    import torch

    from getm_gb300 import _lib
    from oracle.models import seos_buoyancy

    rng = np.random.default_rng(12)
    n = 200_000
    S = rng.uniform(0.0, 40.0, n)
    T = rng.uniform(-2.0, 32.0, n)
    z = rng.uniform(0.0, 6000.0, n)
    rho_ref, b_ref = seos_buoyancy(S, T, z)
    Sd, Td, zd = (torch.from_numpy(a).cuda() for a in (S, T, z))
    rho = torch.empty(n, dtype=torch.float64, device="cuda")
    b = torch.empty_like(rho)
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("getm_density_buoyancy_f64s", n, Sd.data_ptr(), Td.data_ptr(), zd.data_ptr(), rho.data_ptr(),
              b.data_ptr(), s)
    torch.cuda.synchronize()
    drho = np.abs(rho.cpu().numpy() - rho_ref).max()
    db = np.abs(b.cpu().numpy() - b_ref).max()
    print(f"density from FP64 tracers: rho {drho:.2e} kg m-3, buoyancy {db:.2e} m s-2")
    assert drho < 2e-12 and db < 2e-14

    # stratified columns: NN from FP64 tracers, float arithmetic vs FP64
    nz, ny, nx = 30, 40, 50
    plane = nx * ny
    h = torch.from_numpy(rng.uniform(1.0, 20.0, (nz, ny, nx))).cuda()
    p = torch.cumsum(h.flip(0), 0).flip(0) - 0.5 * h
    zc = -p
    temp = (10.0 + 10.0 * torch.exp(zc / 200.0) + 0.01 * torch.from_numpy(rng.standard_normal((nz, ny, nx))).cuda())
    salt = 35.0 + 0.5 * torch.tanh(zc / 300.0)
    mask = torch.from_numpy((rng.random((ny, nx)) > 0.2).astype(np.int32)).cuda()
    nn64 = torch.zeros((nz + 1, ny, nx), dtype=torch.float64, device="cuda")
    nn32 = torch.zeros((nz + 1, ny, nx), dtype=torch.float32, device="cuda")
    _lib.call("getm_buoyancy_frequency", nx, ny, nz, mask.data_ptr(), h.data_ptr(), p.data_ptr(), salt.data_ptr(),
              temp.data_ptr(), nn64.data_ptr(), s)
    _lib.call("getm_buoyancy_frequency_f64s", nx, ny, nz, mask.data_ptr(), h.data_ptr(), p.data_ptr(),
              salt.data_ptr(), temp.data_ptr(), nn32.data_ptr(), s)
    torch.cuda.synchronize()
    wet = mask.bool().cpu().numpy()
    e = rel(host(nn32)[1:-1].astype(np.float64), host(nn64)[1:-1], wet)
    print(f"NN from FP64 tracers in float arithmetic: {e:.2e}")
    assert e < 1e-5
    assert plane > 0
