"""Domain totals (Simulation.totals) against the oracle's numpy sums and the
exactly rounded sum (math.fsum), in both forms; repeated calls are bitwise
identical (fixed reduction order)."""

import math

import numpy as np
import pytest

from tests.gpu_helpers import host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_totals(precision):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation
    from oracle import models

    wl = workloads.seamount(nx=60, ny=44, nz=12, dx=10000.0)
    p = wl.params
    s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision)
    rng = np.random.default_rng(5)
    for tr in (s.temp, s.salt):
        vals = torch.from_numpy(rng.uniform(1e-3, 10.0, tr.all_values.shape)).to(tr.all_values)
        tr.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, vals, tr.all_values))
    s.start(10.0, 10)
    for _ in range(10):
        s.advance()
    vol, trs = s.totals
    again = s.totals_device().clone()
    assert torch.equal(again, s.totals_device())
    T = s.T
    D, hn, area, mask = host(T.D.all_values), host(T.hn.all_values), host(T.area.all_values), host(T.mask.all_values)
    tracers = [host(t.all_values).astype(np.float64) for t in (s.temp, s.salt)]
    ref = models.totals(_Grid(wl.T, mask, area), D, hn, tracers)
    i = (Ellipsis, slice(T.haloy, T.haloy + T.ny), slice(T.halox, T.halox + T.nx))
    wet = mask[i] != 0
    exact = [math.fsum((D * area)[i][wet])]
    for c in tracers:
        exact.append(math.fsum((c * area * hn)[i][:, wet].ravel()))
    got = [vol] + [tot for _, tot, _ in trs]
    for g, r, e in zip(got, ref, exact):
        assert abs(g - e) <= 4e-16 * abs(e)
        assert abs(g - r) <= 1e-12 * abs(r)
    for (t, tot, mean), e in zip(trs, exact[1:]):
        assert mean == pytest.approx(e / exact[0], rel=1e-15)


class _Grid:
    """Minimal grid view for the oracle's totals (interior slice, mask, area)."""

    def __init__(self, hg, mask, area):
        self.mask, self.area = mask, area
        self.interior = (Ellipsis, slice(hg.haloy, hg.haloy + hg.ny), slice(hg.halox, hg.halox + hg.nx))
