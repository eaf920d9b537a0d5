"""Parity of the full split-explicit baroclinic step (GPU Simulation) with the
oracle restatement of pygetm's Simulation/Momentum on a reduced seamount box.

Tolerance: 1e-9 relative to each field's magnitude after several macro steps
(FP64 on both sides; the GPU fuses multiply-adds and sums columns in a
different order, and those last-bit differences are carried through the
dynamics)."""

import numpy as np
import pytest

from tests.test_gpu_operators import close

pytestmark = pytest.mark.gpu


def _pair(nx=40, ny=30, nz=10, dx=10000.0, split=10, internal_pressure="shchepetkin_mcwilliams", runtype=4,
          Am=0.0, An=0.0, coriolis=1, timestep=10.0):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.momentum import CoriolisScheme, Momentum
    from getm_gb300.simulation import Simulation as GS
    from oracle.models import Momentum as OM
    from oracle.models import Simulation as OS

    wl = workloads.seamount(nx=nx, ny=ny, nz=nz, dx=dx)
    p = wl.params
    o = OS(wl.T, wl.dga, runtype=runtype, num=p["num"], nuh=p["nuh"], internal_pressure=internal_pressure,
           momentum=OM(Am=Am, An=An, coriolis_scheme=coriolis))
    g = GS(wl.T, wl.dga, runtype=runtype, num=p["num"], nuh=p["nuh"], internal_pressure=internal_pressure,
           momentum=Momentum(Am=Am, An=An, coriolis_scheme=CoriolisScheme(coriolis)))
    if runtype == 4:
        temp0 = np.where(o.T.mask[None] != 0, workloads.seamount_temperature(o.T.zc), o.temp)
        o.temp[...] = temp0
        g.temp.all_values.copy_(torch.from_numpy(temp0))
    o.start(timestep, split)
    g.start(timestep, split)
    return wl, o, g


def _compare(wl, o, g, rtol):
    T = wl.T
    wetT = T.mask == 1
    wetU = T.ugrid.mask == 1
    wetV = T.vgrid.mask == 1
    h = lambda a: a.all_values.detach().cpu().numpy()  # noqa: E731
    errs = {}
    errs["z"] = close(h(g.T.z), o.T.z, rtol, wetT)
    errs["U"] = close(h(g.momentum.U), o.momentum.U, rtol, wetU)
    errs["V"] = close(h(g.momentum.V), o.momentum.V, rtol, wetV)
    errs["uk"] = close(h(g.momentum.uk), o.momentum.uk, rtol, wetU)
    errs["vk"] = close(h(g.momentum.vk), o.momentum.vk, rtol, wetV)
    errs["ww"] = close(h(g.momentum.ww)[1:-1], o.momentum.ww[1:-1], rtol, wetT)
    errs["hn"] = close(h(g.T.hn), o.T.hn, rtol, wetT)
    if hasattr(o, "temp"):
        errs["temp"] = close(h(g.temp), o.temp, rtol, wetT)
        errs["salt"] = close(h(g.salt), o.salt, rtol, wetT)
        errs["idpdx"] = close(h(g.idpdx), o.idpdx, rtol, wetU)
        errs["idpdy"] = close(h(g.idpdy), o.idpdy, rtol, wetV)
        if o.istep > 0:
            from oracle.models import seos_nsquared

            NN = seos_nsquared(T.mask, o.T.hn, o.depth, o.salt, o.temp)
            errs["NN"] = close(h(g.NN)[1:-1], NN, rtol, wetT)
    if o.istep > 0:
        m, om = g.momentum, o.momentum
        errs["SS"] = close(h(m.SS)[1:-1], om.SS[1:-1], rtol, wetT)
        errs["ustar_b"] = close(h(m.ustar_b), om.ustar_b, rtol, wetT)
        errs["rru"] = close(h(m.rru), om.rru, rtol, wetU)
        errs["SxA"] = close(h(m.SxA), om.SxA, rtol, wetU)
        errs["SxF"] = close(h(m.SxF), om.SxF, rtol, wetU)
        if om._Am_const > 0.0:
            errs["diffU"] = close(h(m.diffU), om.diffU, rtol, wetU)
            errs["diffpk"] = close(h(m.diffpk), om.diffpk, rtol, wetU)
            errs["SxD"] = close(h(m.SxD), om.SxD, rtol, wetU)
        if om.An_uu is not None:
            errs["dampU"] = close(h(m.dampU), om.dampU, rtol, wetU)
            errs["dampV"] = close(h(m.dampV), om.dampV, rtol, wetV)
    return errs


def test_start_matches():
    wl, o, g = _pair()
    _compare(wl, o, g, 1e-11)


@pytest.mark.parametrize("internal_pressure", ["shchepetkin_mcwilliams", "blumberg_mellor"])
def test_macro_steps(internal_pressure):
    wl, o, g = _pair(internal_pressure=internal_pressure)
    for _ in range(30):  # three macro steps of 10 microsteps
        o.advance()
        g.advance()
    errs = _compare(wl, o, g, 1e-9)
    print(errs)


def test_barotropic_3d():
    wl, o, g = _pair(runtype=2)
    for _ in range(20):
        o.advance()
        g.advance()
    _compare(wl, o, g, 1e-9)


@pytest.mark.parametrize("Am,An", [(40.0, 0.0), (0.0, 25.0), (40.0, 25.0)])
def test_momentum_diffusion_and_damping(Am, An):
    """Horizontal momentum diffusion (Am > 0: momentum_diffusion of the 2D and
    3D velocities, momentum.py:1051-1064 and :963-978) and numerical damping
    (An > 0: horizontal_diffusion of the transports, momentum.py:751-758)
    through three macro steps; these configurations run the substep's
    operations one launch each."""
    wl, o, g = _pair(Am=Am, An=An)
    assert g._split2d is None
    for _ in range(30):
        o.advance()
        g.advance()
    print(_compare(wl, o, g, 1e-9))


def test_espelid_coriolis():
    """The ESPELID Coriolis scheme (momentum.py:1136-1142) in 2D and 3D
    through three macro steps."""
    wl, o, g = _pair(coriolis=2)
    assert g._split2d is None
    for _ in range(30):
        o.advance()
        g.advance()
    print(_compare(wl, o, g, 1e-9))
