"""Open boundaries on the GPU against the oracle: a tidal channel with
Flather (elevation), clamped and Flather (transport) elevation boundaries
and zero-gradient, sponge and clamped tracer boundaries.  Tolerance 1e-9
relative to each field's magnitude after several macro steps (as for the
closed seamount)."""

import numpy as np
import pytest

from tests.test_gpu_operators import close

pytestmark = pytest.mark.gpu


def _pair(precision="fp64", fused=True):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation as GS
    from oracle.models import Simulation as OS

    wl = workloads.tidal_channel(nx=40, ny=24, nz=6)
    p = wl.params
    o = OS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    g = GS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, fused_2d=fused)
    temp0 = np.where(o.T.mask[None] != 0, 12.0 + o.T.zc / 10.0, o.temp)
    x0 = o.T.x[o.T.mask != 0].min()
    salt0 = np.where(o.T.mask[None] != 0, 30.0 + 0.01 * (o.T.x[None] - x0) / 1000.0, o.salt)
    o.temp[...] = temp0
    o.salt[...] = salt0
    g.temp.all_values.copy_(torch.from_numpy(temp0))
    g.salt.all_values.copy_(torch.from_numpy(salt0))
    o.start(p["timestep"], p["split_factor"])
    g.start(p["timestep"], p["split_factor"])
    return wl, o, g


@pytest.mark.parametrize("fused", [True, False])
def test_channel_matches_oracle(fused):
    wl, o, g = _pair(fused=fused)
    for _ in range(4 * wl.params["split_factor"]):
        o.advance()
        g.advance()
    T = wl.T
    h = lambda a: a.all_values.detach().cpu().numpy()  # noqa: E731
    water = T.mask != 0
    close(h(g.T.z), o.T.z, 1e-9, water)
    close(h(g.momentum.U), o.momentum.U, 1e-9, T.ugrid.mask != 0)
    close(h(g.momentum.V), o.momentum.V, 1e-9, T.vgrid.mask != 0)
    close(h(g.momentum.uk), o.momentum.uk, 1e-9, T.ugrid.mask != 0)
    close(h(g.temp), o.temp, 1e-9, water)
    close(h(g.salt), o.salt, 1e-9, water)
    assert np.abs(o.T.z[water]).max() > 0.1  # the tide is in


def test_channel_mixed_runs_close_to_fp64():
    import torch

    wl, o, a = _pair("fp64")
    _, _, b = _pair("mixed")
    for _ in range(4 * wl.params["split_factor"]):
        a.advance()
        b.advance()
    torch.cuda.synchronize()
    water = wl.T.mask != 0
    za, zb = a.T.z.all_values.cpu().numpy(), b.T.z.all_values.cpu().numpy()
    assert np.abs(za - zb)[water].max() < 1e-5 * np.abs(za[water]).max()
