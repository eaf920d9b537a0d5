"""Parity of the FP64 GPU path with the oracle at the benchmark
configurations' full sizes.

* Seamount 400 x 300 x 40 (dx = 2 km, dt2d = 4 s, 30 substeps per 3D step):
  the full split-explicit baroclinic step from rest, compared after the
  first and after the second 3D step, field by field (elevation, transports,
  3D velocities, vertical velocity, layer thicknesses, both tracers, both
  internal-pressure gradients, squared buoyancy and shear frequency, bottom
  shear velocity, slow terms).
* Tracer transport 120 x 100 x 30 (dx = 1 km, dt = 30 s, superbee, implicit
  vertical diffusion): 500 steps, the error recorded every 50 steps; the
  drift over the run is bounded.

Tolerances (relative to each field's largest magnitude on water points):
1e-10 after one seamount 3D step and 1e-9 after two (the GPU contracts
multiply-adds and sums columns in its own order; those last-bit differences
pass through the dynamics, where the flow is the small residual of the
sigma-coordinate pressure gradient); 1e-10 for the tracer over all 500
transport steps.
"""

import numpy as np
import pytest

from tests.test_gpu_operators import close

pytestmark = pytest.mark.gpu


def _host(a):
    return a.all_values.detach().cpu().numpy()


def _seamount_errors(wl, o, g):
    """Max relative error of every compared field (no assertion)."""
    from oracle.models import seos_nsquared

    T = wl.T
    wetT, wetU, wetV = T.mask == 1, T.ugrid.mask == 1, T.vgrid.mask == 1
    m, om = g.momentum, o.momentum
    pairs = {
        "z": (g.T.z, o.T.z, wetT), "U": (m.U, om.U, wetU), "V": (m.V, om.V, wetV),
        "uk": (m.uk, om.uk, wetU), "vk": (m.vk, om.vk, wetV), "hn": (g.T.hn, o.T.hn, wetT),
        "temp": (g.temp, o.temp, wetT), "salt": (g.salt, o.salt, wetT),
        "idpdx": (g.idpdx, o.idpdx, wetU), "idpdy": (g.idpdy, o.idpdy, wetV),
        "ustar_b": (m.ustar_b, om.ustar_b, wetT), "SxA": (m.SxA, om.SxA, wetU), "SyA": (m.SyA, om.SyA, wetV),
        "SxB": (m.SxB, om.SxB, wetU), "SxF": (m.SxF, om.SxF, wetU),
    }
    errs = {}
    for name, (a, b, wet) in pairs.items():
        errs[name] = close(_host(a), b, 1.0, wet)
    errs["ww"] = close(_host(m.ww)[1:-1], om.ww[1:-1], 1.0, wetT)
    errs["SS"] = close(_host(m.SS)[1:-1], om.SS[1:-1], 1.0, wetT)
    NN = seos_nsquared(T.mask, o.T.hn, o.depth, o.salt, o.temp)
    errs["NN"] = close(_host(g.NN)[1:-1], NN, 1.0, wetT)
    return errs


def test_seamount_full_size_two_3d_steps():
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation as GS
    from oracle.models import Simulation as OS

    wl = workloads.seamount()  # 400 x 300 x 40
    assert (wl.T.nx, wl.T.ny, wl.T.nz) == (400, 300, 40)
    p = wl.params
    o = OS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    g = GS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    temp0 = np.where(o.T.mask[None] != 0, workloads.seamount_temperature(o.T.zc), o.temp)
    o.temp[...] = temp0
    g.temp.all_values.copy_(torch.from_numpy(temp0))
    o.start(p["timestep"], p["split_factor"])
    g.start(p["timestep"], p["split_factor"])
    assert g._split2d is not None  # the one-launch substep is on the path
    for step, rtol in ((1, 1e-10), (2, 1e-9)):
        for _ in range(p["split_factor"]):
            o.advance()
            g.advance()
        torch.cuda.synchronize()
        assert g.split2d_status() == 0
        errs = _seamount_errors(wl, o, g)
        print(f"seamount 400x300x40, after 3D step {step}: "
              + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
        bad = {k: v for k, v in errs.items() if not v <= rtol}
        assert not bad, f"3D step {step}: above {rtol}: {bad}"


def test_tracer_transport_full_size_500_steps():
    from getm_gb300 import workloads
    from getm_gb300.simulation import TracerTransport as GT
    from oracle.models import TracerTransport as OT

    wl = workloads.tracer_transport()  # 120 x 100 x 30
    assert (wl.T.nx, wl.T.ny, wl.T.nz) == (120, 100, 30)
    g = GT(wl)
    o = OT(wl)
    wet = wl.T.mask == 1
    series = []
    for n in range(1, 501):
        g.step()
        o.step()
        if n % 50 == 0:
            series.append((n, close(_host(g.tracers[0]), o.tracers[0], 1.0, wet)))
    print("tracer transport 120x100x30, relative error every 50 steps: "
          + ", ".join(f"{n}: {e:.2e}" for n, e in series))
    worst = max(e for _, e in series)
    assert worst <= 1e-10, series
    # the tracer stays bounded like the oracle's (no growth of the blob)
    a = _host(g.tracers[0])[..., wet]
    b = o.tracers[0][..., wet]
    assert a.max() <= b.max() * (1 + 1e-12) + 1e-300 and a.min() >= b.min() - 1e-12
