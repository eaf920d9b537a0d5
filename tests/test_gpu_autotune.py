"""Launch shapes change no result: a simulation run with other shapes of the
x pass, the 3D y pass, the column kernels and the one-launch substep ends in
bitwise the same state; and the tuner runs end to end on a small domain."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(tiles, precision):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount(nx=64, ny=48, nz=8, dx=8000.0)
    p = wl.params
    s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, tiles=tiles)
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                        s.temp.all_values.double()))
    s.start(10.0, 7)
    for _ in range(2 * 7 + 3):
        s.advance()
    torch.cuda.synchronize()
    assert s.split2d_status() == 0
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_shapes_change_no_result(precision):
    import torch

    from getm_gb300 import autotune, checkpoint

    other = {"xpass_rows": 2, "ymarch_chunk": 16, "column_rows": 1, "substep_blocks_per_sm": 1, "xpass_vec": 0}
    a = _run(autotune.DEFAULTS, precision)
    b = _run(other, precision)
    autotune.apply(None)
    sa, sb = checkpoint.state_tensors(a), checkpoint.state_tensors(b)
    bad = [k for k in sa if not bool(((sa[k] == sb[k]) | (torch.isnan(sa[k]) & torch.isnan(sb[k]))).all())]
    assert not bad, bad[:10]


def test_tune_small_member():
    from getm_gb300 import autotune, workloads
    from getm_gb300.ensemble import make_member

    wl = workloads.ensemble_member(np.random.default_rng(3), nmin=64, nmax=64, nzmin=10, nzmax=10)
    sim = make_member(wl, "mixed")
    best, t, t0, trials = autotune.tune(sim, rounds=1, replays=2)
    assert set(best) == set(autotune.KNOBS) and t <= t0 and len(trials) >= 5
    assert autotune.current() == autotune.DEFAULTS


@pytest.mark.parametrize("nx", [40, 256, 300, 301])
@pytest.mark.parametrize("storage", ["float32", "float64"])
@pytest.mark.parametrize("ntracer", [1, 3])
def test_xpass_forms_bitwise(nx, storage, ntracer):
    """The 3D x pass with four cells per lane (rows swept in chunks of 128
    cells: one partial chunk, several, a partial last one; nx_ = 305 not a
    multiple of four, so one cell per lane) against one cell per lane:
    mixed-form advection of one or three fields (a pair and a single) with
    horizontal diffusion, bit for bit."""
    import torch

    from getm_gb300 import autotune, operators
    from getm_gb300.core import CENTERS, INTERFACES, Array
    from tests.gpu_helpers import dev
    from tests.test_gpu_operators import setup, velocity

    Th, To, Td, rng = setup(seed=nx + ntracer, nx=nx, ny=20, nz=6)
    nz = Th.nz
    u = velocity(Th.ugrid, rng, nz, 0.3)
    v = velocity(Th.vgrid, rng, nz, 0.3)
    w = rng.uniform(-5e-4, 5e-4, (nz + 1, Th.ny_, Th.nx_))
    w[0] = w[-1] = 0.0
    Ahu = rng.uniform(0.0, 50.0, (Th.ny_, Th.nx_))
    Ahv = rng.uniform(0.0, 50.0, (Th.ny_, Th.nx_))
    tr = [rng.uniform(5.0, 10.0, (nz, Th.ny_, Th.nx_)) for _ in range(ntracer)]
    dt = torch.float32 if storage == "float32" else torch.float64
    f32 = lambda g, a, z: Array(g, dev(a).float(), z=z)  # noqa: E731
    out = []
    for vec in (1, 0):
        autotune.apply({"xpass_vec": vec})
        ad = operators.Advection(Td, operators.AdvectionScheme(5))
        trd = [Array(Td, dev(t).to(dt), z=CENTERS) for t in tr]
        ad.apply_3d_batch(f32(Td.ugrid, u, CENTERS), f32(Td.vgrid, v, CENTERS), f32(Td, w, INTERFACES), 600.0, trd,
                          Ah_u=Array(Td.ugrid, dev(Ahu)), Ah_v=Array(Td.vgrid, dev(Ahv)))
        torch.cuda.synchronize()
        out.append([t.all_values.clone() for t in trd] + [ad.h.clone()])
    autotune.apply(None)
    for a, b in zip(*out):
        assert torch.equal(a, b)
