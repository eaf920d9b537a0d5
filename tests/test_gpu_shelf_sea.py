"""The many-tracer shelf sea (fractal bathymetry, ~35 % land, tidal open
boundaries, an initial non-divergent flow and passive tracers) on a reduced
grid: FP64 GPU against the oracle (1e-9 of each field's magnitude), and the
mixed form's tracer errors against FP64."""

import numpy as np
import pytest

from tests.test_gpu_operators import close

pytestmark = pytest.mark.gpu


def _oracle(wl):
    from oracle.models import Simulation as OS

    p = wl.params
    o = OS(wl.T, wl.dga, runtype=2, num=p["num"], nuh=p["nuh"])
    for f in p["tracers"]:
        o.tracers.append(np.broadcast_to(f, (wl.T.nz,) + f.shape).copy())
        o.molecular.append(0.0)
    m = o.momentum
    for tp2, tp3, g, src in ((m.U, m.pk, o.U, p["U"]), (m.V, m.qk, o.V, p["V"])):
        tp2[...] = src
        with np.errstate(all="ignore"):
            frac = np.where(g.D > 0, g.hn / g.D, 0.0)
        tp3[...] = src * frac
    o.start(p["timestep"], p["split_factor"])
    return o


def test_shelf_sea_matches_oracle():
    from getm_gb300 import workloads

    wl = workloads.shelf_sea(nx=96, ny=80, nz=6, ntracer=3)
    o = _oracle(wl)
    g = workloads.start_shelf_sea(wl, "fp64")
    for _ in range(3 * wl.params["split_factor"]):
        o.advance()
        g.advance()
    T = wl.T
    h = lambda a: a.all_values.detach().cpu().numpy()  # noqa: E731
    water = T.mask != 0
    close(h(g.T.z), o.T.z, 1e-9, water)
    close(h(g.momentum.U), o.momentum.U, 1e-9, T.ugrid.mask != 0)
    for a, b in zip(g.tracers._tracers, o.tracers):
        close(h(a), b, 1e-9, water)


def test_shelf_sea_mixed_tracers():
    import torch

    from getm_gb300 import workloads

    wl = workloads.shelf_sea(nx=96, ny=80, nz=6, ntracer=3)
    a = workloads.start_shelf_sea(wl, "fp64")
    b = workloads.start_shelf_sea(wl, "mixed")
    for _ in range(5 * wl.params["split_factor"]):
        a.advance()
        b.advance()
    torch.cuda.synchronize()
    water = torch.from_numpy(wl.T.mask == 1).cuda()
    for x, y in zip(a.tracers._tracers, b.tracers._tracers):
        xa, ya = x.all_values[..., water], y.all_values.double()[..., water]
        assert float((xa - ya).abs().max() / xa.abs().max()) < 1e-5
    ta, tb = a.totals_device(), b.totals_device()
    assert float(((ta - tb).abs() / ta.abs()).max()) < 1e-5
