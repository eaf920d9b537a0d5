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


def _oracle(wl, runtype=4, internal_pressure="shchepetkin_mcwilliams", Am=0.0, An=0.0, coriolis=1, timestep=10.0,
            split=10):
    from getm_gb300 import workloads
    from oracle.models import Momentum as OM
    from oracle.models import Simulation as OS

    p = wl.params
    o = OS(wl.T, wl.dga, runtype=runtype, num=p["num"], nuh=p["nuh"], internal_pressure=internal_pressure,
           momentum=OM(Am=Am, An=An, coriolis_scheme=coriolis))
    if runtype == 4:
        o.temp[...] = np.where(o.T.mask[None] != 0, workloads.seamount_temperature(o.T.zc), o.temp)
        o.temp0 = o.temp.copy()
    o.start(timestep, split)
    return o


def _spread_run(wl, nadvance, **kw):
    """Fields of the oracle built with and without contracted multiply-adds
    after ``nadvance`` advances, and their relative differences."""
    from tests.gpu_helpers import oracle_variant, relative_errors

    runs, temp0 = [], None
    for variant in ("serial", "fma"):
        with oracle_variant(variant):
            o = _oracle(wl, **kw)
            if temp0 is None:
                temp0 = o.temp0
            for _ in range(nadvance):
                o.advance()
            runs.append(_oracle_fields(wl, o))
    return runs[0], relative_errors(runs[1], runs[0]), temp0


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


def _oracle_fields(wl, o):
    """The compared fields of an oracle simulation, name -> (array, water mask)."""
    from oracle.models import seos_nsquared

    T = wl.T
    wT, wU, wV = T.mask == 1, T.ugrid.mask == 1, T.vgrid.mask == 1
    om = o.momentum
    f = {"z": (o.T.z, wT), "U": (om.U, wU), "V": (om.V, wV), "uk": (om.uk, wU), "vk": (om.vk, wV),
         "ww": (om.ww[1:-1], wT), "hn": (o.T.hn, wT)}
    if hasattr(o, "temp"):
        f.update(temp=(o.temp, wT), salt=(o.salt, wT), idpdx=(o.idpdx, wU), idpdy=(o.idpdy, wV))
        if o.istep > 0:
            f["NN"] = (seos_nsquared(T.mask, o.T.hn, o.depth, o.salt, o.temp), wT)
    if o.istep > 0:
        f.update(SS=(om.SS[1:-1], wT), ustar_b=(om.ustar_b, wT), rru=(om.rru, wU), SxA=(om.SxA, wU),
                 SxB=(om.SxB, wU), SxF=(om.SxF, wU))
        if om._Am_const > 0.0:
            f.update(diffU=(om.diffU, wU), diffpk=(om.diffpk, wU))
        if om.An_uu is not None:
            f.update(dampU=(om.dampU, wU), dampV=(om.dampV, wV))
    out = {k: (np.array(v, copy=True), m) for k, (v, m) in f.items()}
    if o.istep > 0 and om._Am_const > 0.0:
        # SxD = sum_k diffpk - diffU(Ui): the small difference of the 3D and
        # 2D diffusion terms, measured against the size of those terms
        scale = float(np.abs(om.diffpk.sum(axis=0)[wU]).max())
        out["SxD"] = (np.array(om.SxD, copy=True), wU, scale)
    return out


def _gpu_fields(g, like):
    """The same fields of a GPU simulation (keys of ``like``)."""
    h = lambda a: a.all_values.detach().cpu().numpy()  # noqa: E731
    m = g.momentum
    src = {"z": h(g.T.z), "U": h(m.U), "V": h(m.V), "uk": h(m.uk), "vk": h(m.vk), "ww": h(m.ww)[1:-1],
           "hn": h(g.T.hn)}
    if hasattr(g, "temp") and g.runtype == 4:
        src.update(temp=h(g.temp), salt=h(g.salt), idpdx=h(g.idpdx), idpdy=h(g.idpdy), NN=h(g.NN)[1:-1])
    for n in ("ustar_b", "rru", "SxA", "SxB", "SxF", "diffU", "SxD", "dampU", "dampV"):
        if n in like:
            src[n] = h(getattr(m, n))
    if "SS" in like:
        src["SS"] = h(m.SS)[1:-1]
    if "diffpk" in like:
        src["diffpk"] = h(m.diffpk)
    return {k: (src[k].astype(np.float64),) + tuple(like[k][1:]) for k in like}


# Tolerance of a field after several split-explicit steps: the GPU's
# difference from the oracle built without contraction may be at most
# FMA_FACTOR times the difference between that oracle and the same oracle
# built with contracted multiply-adds (the reference's own spread between
# two valid compilations: gfortran contracts on aarch64, not on x86-64),
# and never more than CAP.  The GPU contracts at more sites than the C
# oracle (also where the oracle's numpy orchestration cannot), hence the
# factor.  Below FLOOR every difference passes.
FMA_FACTOR = 100.0
FLOOR = 1e-12
CAP = 1e-5


def check_against_spread(gpu_err: dict, spread: dict, floor=FLOOR, factor=FMA_FACTOR, cap=CAP):
    bad = {k: (e, spread[k]) for k, e in gpu_err.items()
           if not (e <= max(floor, factor * spread[k]) and e <= cap)}
    assert not bad, f"(gpu error, oracle FMA spread) above bound: {bad}"


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


def _gpu_vs_spread(nadvance=30, **kw):
    """GPU error after ``nadvance`` advances against the oracle's FMA spread."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.momentum import CoriolisScheme, Momentum
    from getm_gb300.simulation import Simulation as GS
    from tests.gpu_helpers import relative_errors

    wl = workloads.seamount(nx=40, ny=30, nz=10, dx=10000.0)
    ref, spread, temp0 = _spread_run(wl, nadvance, **kw)
    p = wl.params
    g = GS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"],
           momentum=Momentum(Am=kw.get("Am", 0.0), An=kw.get("An", 0.0),
                             coriolis_scheme=CoriolisScheme(kw.get("coriolis", 1))))
    g.temp.all_values.copy_(torch.from_numpy(temp0))
    g.start(10.0, 10)
    for _ in range(nadvance):
        g.advance()
    torch.cuda.synchronize()
    err = relative_errors(_gpu_fields(g, ref), ref)
    print("gpu error / oracle FMA spread: "
          + ", ".join(f"{k} {err[k]:.1e}/{spread[k]:.1e}" for k in err))
    return g, err, spread


@pytest.mark.parametrize("Am,An", [(40.0, 0.0), (0.0, 25.0), (40.0, 25.0)])
def test_momentum_diffusion_and_damping(Am, An):
    """Horizontal momentum diffusion (Am > 0: momentum_diffusion of the 2D and
    3D velocities, momentum.py:1051-1064 and :963-978) and numerical damping
    (An > 0: horizontal_diffusion of the transports, momentum.py:751-758)
    through three macro steps; these configurations run the substep's
    operations one launch each."""
    g, err, spread = _gpu_vs_spread(Am=Am, An=An)
    assert g._split2d is None
    check_against_spread(err, spread, floor=1e-9)


def test_espelid_coriolis():
    """The ESPELID Coriolis scheme (momentum.py:1136-1142) in 2D and 3D
    through three macro steps."""
    g, err, spread = _gpu_vs_spread(coriolis=2)
    assert g._split2d is None
    check_against_spread(err, spread, floor=1e-9)
