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


def _pair(nx=40, ny=30, nz=10, dx=10000.0, split=10, internal_pressure="shchepetkin_mcwilliams", runtype=4):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation as GS
    from oracle.models import Simulation as OS

    wl = workloads.seamount(nx=nx, ny=ny, nz=nz, dx=dx)
    p = wl.params
    o = OS(wl.T, wl.dga, runtype=runtype, num=p["num"], nuh=p["nuh"], internal_pressure=internal_pressure)
    g = GS(wl.T, wl.dga, runtype=runtype, num=p["num"], nuh=p["nuh"], internal_pressure=internal_pressure)
    if runtype == 4:
        temp0 = np.where(o.T.mask[None] != 0, workloads.seamount_temperature(o.T.zc), o.temp)
        o.temp[...] = temp0
        g.temp.all_values.copy_(torch.from_numpy(temp0))
    o.start(10.0, split)
    g.start(10.0, split)
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
        if o.istep > 0:
            from oracle.models import seos_nsquared

            NN = seos_nsquared(T.mask, o.T.hn, o.depth, o.salt, o.temp)
            errs["NN"] = close(h(g.NN)[1:-1], NN, rtol, wetT)
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
