"""The k-epsilon closure on the GPU (getm_keps_advance) against its CPU
restatement (oracle/turbulence.py) on random columns, FP64 (within 100 times
the oracle's own response to a 2-ulp input perturbation: the GPU contracts
multiply-adds) and with float NN, SS, num, nuh (1e-5); a wind-driven,
stratified tidal channel with the closure against the oracle simulation;
and a wind-driven simulation with the closure: finite, positive viscosity,
and the same state, bit for bit, with the 3D step on one stream or
three."""

import numpy as np
import pytest

from tests.gpu_helpers import dev, host
from tests.test_gpu_operators import close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_keps_matches_oracle(dtype):
    import torch

    from getm_gb300.core import INTERFACES, Array, make_grids
    from getm_gb300.vertical_mixing import GOTM
    from oracle import turbulence as K
    from tests.helpers import full_grid

    Th, rng = full_grid(nx=40, ny=30, nz=20, seed=5)
    Td = make_grids(Th)
    nz = Th.nz
    shape = (nz + 1, Th.ny_, Th.nx_)
    h = np.where(Th.mask[None] != 0, rng.uniform(0.5, 3.0, (nz, Th.ny_, Th.nx_)), 1.0)
    Td.hn.all_values.copy_(torch.from_numpy(h))
    NN = rng.uniform(-1e-5, 1e-4, shape)
    SS = rng.uniform(0.0, 1e-3, shape)
    us = rng.uniform(0.0, 0.02, (Th.ny_, Th.nx_))
    ub = rng.uniform(0.0, 0.02, (Th.ny_, Th.nx_))
    z0s = np.full((Th.ny_, Th.nx_), 0.1)
    z0b = rng.uniform(0.001, 0.01, (Th.ny_, Th.nx_))
    if dtype == "float32":
        NN, SS = (x.astype(np.float32).astype(np.float64) for x in (NN, SS))
    td = torch.float64 if dtype == "float64" else torch.float32
    vm = GOTM()
    vm.initialize(Td, dtype=td)
    # developed turbulence to start from, the same on both sides
    k0 = rng.uniform(1e-6, 1e-4, shape)
    e0 = rng.uniform(1e-9, 1e-7, shape)
    cmu = vm.params.cm0 ** 4
    nu0 = cmu * k0 * k0 / e0
    if dtype == "float32":
        nu0 = nu0.astype(np.float32).astype(np.float64)
    vm.tke.all_values.copy_(torch.from_numpy(k0))
    vm.eps.all_values.copy_(torch.from_numpy(e0))
    vm.num.all_values.copy_(torch.from_numpy(nu0))
    vm.nuh.all_values.copy_(torch.from_numpy(nu0))
    o = {n: x.copy() for n, x in dict(tke=k0, eps=e0, L=np.zeros(shape), num=nu0, nuh=nu0.copy()).items()}

    def arr(x, z):
        return Array(Td, dev(x).to(td) if z else dev(x), z=z)

    # the same oracle run from a viscosity perturbed by two units in the last
    # place: these random columns (unstable, strongly sheared) grow k by up to
    # six orders of magnitude in five steps, which amplifies last-bit
    # differences such as the GPU's contracted multiply-adds
    p = {n: x.copy() for n, x in o.items()}
    p["num"] = p["num"] * (1.0 + 4.4e-16)
    for _ in range(5):
        vm.advance(600.0, arr(us, False), arr(ub, False), arr(z0s, False), arr(z0b, False), arr(NN, INTERFACES),
                   arr(SS, INTERFACES))
        for st in (o, p):
            K.keps_advance(Th, 600.0, h, us, ub, z0s, z0b, NN, SS, st["tke"], st["eps"], st["L"], st["num"],
                           st["nuh"])
            if dtype == "float32":  # the stored viscosities are float on the GPU
                st["num"] = st["num"].astype(np.float32).astype(np.float64)
                st["nuh"] = st["nuh"].astype(np.float32).astype(np.float64)
    torch.cuda.synchronize()
    sel = np.zeros((Th.ny_, Th.nx_), dtype=bool)
    sel[2:-2, 2:-2] = Th.mask[2:-2, 2:-2] == 1
    for n in ("tke", "eps", "L", "num", "nuh"):
        a, b = o[n][:, sel], p[n][:, sel]
        spread = float(np.abs(a - b).max() / np.abs(a).max())
        # FP64: 100 times the oracle's own response to the perturbation (at
        # least 1e-12); float NN, SS, num and nuh: 1e-5
        rtol = max(1e-12, 100.0 * spread) if dtype == "float64" else 1e-5
        e = close(host(getattr(vm, n).all_values).astype(np.float64), o[n], rtol, sel)
        print(f"{n}: {e:.2e} (oracle 2-ulp spread {spread:.1e})")


def _member_sim(concurrent, precision="fp64"):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Fluxes, Simulation
    from getm_gb300.vertical_mixing import GOTM

    wl = workloads.ensemble_member(np.random.default_rng(8), nmin=40, nmax=40, nzmin=12, nzmax=12)
    p = wl.params
    s = Simulation(wl.T, wl.dga, precision=precision, airsea=Fluxes(taux=max(p.get("taux", 0.0), 0.1)),
                   vertical_mixing=GOTM(), concurrent_3d=concurrent)
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 20.0 + p.get("dT", 10.0) * zc / 100.0,
                                        s.temp.all_values.double()))
    s.start(p["timestep"], p["split_factor"])
    for _ in range(4 * s.split_factor):
        s.advance()
    torch.cuda.synchronize()
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_simulation_with_keps(precision):
    import torch

    a = _member_sim(True, precision)
    b = _member_sim(False, precision)
    wet = a.T.mask.all_values == 1
    num = a.vertical_mixing.num.all_values[:, wet].double()
    assert torch.isfinite(num).all() and (num > 0).all()
    assert float(a.vertical_mixing.tke.all_values[:, wet].max()) > 1e-8  # the wind has stirred the water
    for n in ("tke", "eps", "num", "nuh"):
        x, y = getattr(a.vertical_mixing, n).all_values, getattr(b.vertical_mixing, n).all_values
        assert bool(((x == y) | (torch.isnan(x) & torch.isnan(y))).all()), n
    assert bool((a.temp.all_values == b.temp.all_values).all())


def _channel_keps_oracle(nadvance):
    """Oracle tidal channel (open boundaries, stratified, wind) with the
    k-epsilon closure from developed turbulence, built with and without
    contracted multiply-adds: fields of the first and the relative spread."""
    from tests.gpu_helpers import oracle_variant, relative_errors

    runs = []
    for variant in ("serial", "fma"):
        with oracle_variant(variant):
            o = _channel(None)
            for _ in range(nadvance):
                o.advance()
            runs.append(_fields(o, o.T.mask))
    return runs[0], relative_errors(runs[1], runs[0])


K0, E0 = 1e-4, 1e-7  # developed turbulence at the start (num = cmu k^2 / eps = 9e-3)


def _channel(precision):
    """The channel with the closure: the oracle (precision None) or a GPU
    simulation of that precision."""
    from getm_gb300 import workloads
    from oracle.models import FILL

    wl = workloads.tidal_channel(nx=40, ny=24, nz=6)
    p = wl.params
    mask = wl.T.mask
    temp0 = lambda zc, t: np.where(mask[None] != 0, 12.0 + zc / 10.0, t)  # noqa: E731
    nu0 = 0.5477 ** 4 * K0 * K0 / E0
    dev_state = {n: np.where(mask[None] != 0, v, FILL) * np.ones((wl.T.nz + 1, 1, 1))
                 for n, v in (("tke", K0), ("eps", E0), ("num", nu0), ("nuh", nu0))}
    if precision is None:
        from oracle.models import Simulation as OS

        o = OS(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], taux=0.2, keps={})
        o.temp[...] = temp0(o.T.zc, o.temp)
        for n, v in dev_state.items():
            getattr(o, n)[...] = v
        o.start(p["timestep"], p["split_factor"])
        return o
    import torch

    from getm_gb300.simulation import Fluxes, Simulation
    from getm_gb300.vertical_mixing import GOTM

    g = Simulation(wl.T, wl.dga, precision=precision, airsea=Fluxes(taux=0.2), vertical_mixing=GOTM())
    zc = host(g.T.zc.all_values).astype(np.float64)
    t = torch.from_numpy(temp0(zc, host(g.temp.all_values).astype(np.float64)))
    g.temp.all_values.copy_(t.to(g.temp.all_values.dtype))
    vm = g.vertical_mixing
    for n, v in dev_state.items():
        a = getattr(vm, n).all_values
        a.copy_(torch.from_numpy(v).to(a.dtype))
    g.start(p["timestep"], p["split_factor"])
    return g


def _fields(s, mask):
    """tke, eps, num (interior interfaces), elevation, velocities and
    temperature of a simulation (oracle or GPU), with their water masks."""
    if hasattr(s, "vertical_mixing"):
        h = lambda a: host(a.all_values).astype(np.float64)  # noqa: E731
        vm, m = s.vertical_mixing, s.momentum
        src = dict(tke=h(vm.tke), eps=h(vm.eps), num=h(vm.num), z=h(s.T.z), uk=h(m.uk), temp=h(s.temp))
        umask = s.U.mask.all_values.cpu().numpy()
    else:
        src = dict(tke=s.tke, eps=s.eps, num=s.num, z=s.T.z, uk=s.momentum.uk, temp=s.temp)
        umask = s.U.mask
    wT, wU = mask == 1, umask == 1
    out = {}
    for n, a in src.items():
        a = a[1:-1] if n in ("tke", "eps", "num") else a
        out[n] = (np.array(a, copy=True), wU if n == "uk" else wT)
    return out


def test_channel_keps_matches_oracle():
    """The closure inside the FP64 split-explicit step of a wind-driven,
    stratified tidal channel with open boundaries (num taken from the
    nearest interior point there) over eight 3D steps: the GPU's difference
    from the oracle against the oracle's own spread between builds with and
    without contracted multiply-adds."""
    import torch

    from tests.gpu_helpers import relative_errors
    from tests.test_gpu_simulation import check_against_spread

    nadvance = 80
    ref, spread = _channel_keps_oracle(nadvance)
    g = _channel("fp64")
    for _ in range(nadvance):
        g.advance()
    torch.cuda.synchronize()
    err = relative_errors(_fields(g, g.T.mask.all_values.cpu().numpy()), ref)
    print("gpu error / oracle FMA spread: " + ", ".join(f"{k} {err[k]:.1e}/{spread[k]:.1e}" for k in err))
    check_against_spread(err, spread, floor=1e-9)
    # the closure is active: interior turbulence has decayed well below its
    # initial level and stays well above the minimum
    tke = ref["tke"][0][:, ref["tke"][1]]
    assert np.median(tke) < 0.1 * K0 and tke.min() > 100 * 1e-10
