"""Parity of the FP64 GPU path with the oracle at the benchmark
configurations' full sizes.

* Seamount 400 x 300 x 40 (dx = 2 km, dt2d = 4 s, 30 substeps per 3D step):
  the full split-explicit baroclinic step from rest, compared after the
  first and after the second 3D step, field by field (elevation, transports,
  3D velocities, vertical velocity, layer thicknesses, both tracers, both
  internal-pressure gradients, squared buoyancy and shear frequency, bottom
  shear velocity and drag, slow terms).
* Tracer transport 120 x 100 x 30 (dx = 1 km, dt = 30 s, superbee, implicit
  vertical diffusion): 500 steps, the error recorded every 50 steps; the
  drift over the run is bounded.

Tolerances (relative to each field's largest magnitude on water points).
Tracers and layer thicknesses: 1e-13 after each seamount 3D step; the
tracer-transport tracer: 1e-12 over all 500 steps.  The seamount's flow
fields (elevation, transports, velocities, w, the internal-pressure
gradient and the terms built from them) are the small residual of large
cancelling terms (the sigma-coordinate pressure gradient over a 4000 m
seamount), so one-ulp differences grow far beyond 1e-12 there: the same
oracle compiled with and without contracted multiply-adds (both valid
builds of the reference; gfortran contracts on aarch64) already differs by
up to 2e-7 (internal-pressure gradient) after one 3D step.  Each such field
must stay within 100 times that spread of the reference itself, and below
1e-5.
"""

import numpy as np
import pytest

from tests.test_gpu_operators import close
from tests.test_gpu_simulation import _gpu_fields, _oracle_fields, check_against_spread

pytestmark = pytest.mark.gpu


def _host(a):
    return a.all_values.detach().cpu().numpy()


def test_seamount_full_size_two_3d_steps():
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation as GS
    from oracle.models import Simulation as OS
    from tests.gpu_helpers import oracle_variant, relative_errors

    wl = workloads.seamount()  # 400 x 300 x 40
    assert (wl.T.nx, wl.T.ny, wl.T.nz) == (400, 300, 40)
    p = wl.params
    nstep = 2
    snaps, temp0 = {}, None
    for variant in ("serial", "fma"):
        with oracle_variant(variant):
            o = OS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
            if temp0 is None:
                temp0 = np.where(o.T.mask[None] != 0, workloads.seamount_temperature(o.T.zc), o.temp)
            o.temp[...] = temp0
            o.start(p["timestep"], p["split_factor"])
            snaps[variant] = []
            for _ in range(nstep):
                for _ in range(p["split_factor"]):
                    o.advance()
                snaps[variant].append(_oracle_fields(wl, o))
            del o
    g = GS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    g.temp.all_values.copy_(torch.from_numpy(temp0))
    g.start(p["timestep"], p["split_factor"])
    assert g._split2d is not None  # the one-launch substep is on the path
    for step in range(nstep):
        for _ in range(p["split_factor"]):
            g.advance()
        torch.cuda.synchronize()
        assert g.split2d_status() == 0
        ref = snaps["serial"][step]
        spread = relative_errors(snaps["fma"][step], ref)
        err = relative_errors(_gpu_fields(g, ref), ref)
        print(f"seamount 400x300x40, 3D step {step + 1}, gpu error / oracle FMA spread: "
              + ", ".join(f"{k} {err[k]:.1e}/{spread[k]:.1e}" for k in err))
        for k in ("temp", "salt", "hn"):
            assert err[k] <= 1e-13, (k, err[k])
        check_against_spread(err, spread)


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
    assert worst <= 1e-12, series
    # the tracer stays bounded like the oracle's (no growth of the blob)
    a = _host(g.tracers[0])[..., wet]
    b = o.tracers[0][..., wet]
    assert a.max() <= b.max() * (1 + 1e-12) + 1e-300 and a.min() >= b.min() - 1e-12
