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

    other = {"xpass_rows": 2, "ymarch_chunk": 16, "column_rows": 1, "substep_blocks_per_sm": 1}
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
