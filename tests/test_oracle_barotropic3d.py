"""Pins the oracle's split-explicit 3D step with the invariants of
python/tests/test_3d_barotropic.py:26-147: in a closed 50 m deep box driven
by a uniform wind (with and without bottom friction), the 3D transports
that the macro step produces satisfy discrete continuity with the vertical
velocity and the change of the layer thicknesses (the "missing vertical
velocity" is zero to rounding, as the reference asserts with check_zero),
an advected tracer's total is conserved and so is the total volume.  Here
the tracer is a randomly perturbed salinity carried by the step's own
advection."""

import numpy as np
import pytest

from getm_gb300.domain import calculate_sigma, create_cartesian


@pytest.mark.parametrize("taux,tauy", [(0.1, -0.1), (-0.1, 0.0), (0.0, 0.1)])
@pytest.mark.parametrize("friction", [True, False])
def test_continuity_and_conservation(taux, tauy, friction):
    from oracle.models import Simulation

    nx, ny, nz = 40, 16, 20
    dom = create_cartesian(500.0 * np.arange(nx), 500.0 * np.arange(ny), f=0.0, H=50.0,
                           z0=0.01 if friction else 0.0)
    T = dom.create_grids(nz, halox=2, haloy=2, velocity_grids=2)
    s = Simulation(T, calculate_sigma(nz), num=1e-3, nuh=1e-3, taux=taux, tauy=tauy)
    Tg, m = s.T, s.momentum
    U, V = Tg.ugrid, Tg.vgrid
    wet = Tg.mask == 1
    rng = np.random.default_rng(7)
    s.salt[:, wet] = 35.0 + 0.5 * rng.random((nz, int(wet.sum())))
    split = 10
    s.start(10.0, split)
    salt0 = (s.salt * Tg.hn)[:, wet].sum()
    vol0 = Tg.z[wet].sum()
    for step in range(1, 8 * split + 1):
        s.advance()
        if step % split:
            continue
        # test_3d_barotropic.py:88-112, halos of 2 dropped
        U1, U2 = (m.pk * U.dy)[:, 2:-2, 1:-3], (m.pk * U.dy)[:, 2:-2, 2:-2]
        V1, V2 = (m.qk * V.dx)[:, 1:-3, 2:-2], (m.qk * V.dx)[:, 2:-2, 2:-2]
        W1, W2 = (m.ww * Tg.area)[:-1, 2:-2, 2:-2], (m.ww * Tg.area)[1:, 2:-2, 2:-2]
        dH = ((Tg.hn - Tg.ho) * Tg.area)[:, 2:-2, 2:-2] / s.macrotimestep
        div = U1 - U2 + V1 - V2 + W1 - W2 - dH
        missing_w = np.abs(div / Tg.area[2:-2, 2:-2])[:, wet[2:-2, 2:-2]].max()
        assert missing_w < 1e-14, (step, missing_w)
    assert np.abs(m.U).max() > 1e-3  # the wind drives a flow
    salt = (s.salt * Tg.hn)[:, wet].sum()
    assert abs(salt - salt0) / salt0 < 1e-13
    assert abs(Tg.z[wet].sum() - vol0) < 1e-12
