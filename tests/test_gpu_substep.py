"""The one-launch 2D substep (getm_split2d_substep): the same state, bit for
bit, as the substep's operations launched one by one, in both forms, eagerly
and replayed from a CUDA graph; its grid barriers never give up."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    import torch

    from getm_gb300 import checkpoint

    sa, sb = checkpoint.state_tensors(a), checkpoint.state_tensors(b)
    return [k for k in sa if not bool(((sa[k] == sb[k]) | (torch.isnan(sa[k]) & torch.isnan(sb[k]))).all())]


def _member(precision, substep_kernel, n3d=4, seed=3):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.ensemble import make_member

    wl = workloads.ensemble_member(np.random.default_rng(seed), nmin=40, nmax=48, nzmin=6, nzmax=8)
    s = make_member(wl, precision, substep_kernel=substep_kernel)
    assert (s._split2d is not None) == substep_kernel
    for _ in range(n3d * s.split_factor):
        s.advance()
    torch.cuda.synchronize()
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_substep_kernel_is_bitwise(precision):
    """A wind-driven member (currents, Coriolis, friction and advection all
    active) after four 3D steps."""
    a, b = _member(precision, True), _member(precision, False)
    assert a.split2d_status() == 0
    bad = _same(a, b)
    assert not bad, bad[:12]
    assert float(a._time) == float(b._time)


def test_substep_kernel_seamount_bitwise():
    """The seamount (density-driven flow over steep bathymetry, odd split
    factor so both momentum orders meet the 3D step)."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    def run(kernel):
        wl = workloads.seamount(nx=40, ny=30, nz=8, dx=10000.0)
        p = wl.params
        s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision="fp64", substep_kernel=kernel)
        zc = s.T.zc.all_values
        s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                            s.temp.all_values))
        s.start(10.0, 7)
        for _ in range(3 * 7 + 3):
            s.advance()
        torch.cuda.synchronize()
        return s

    a, b = run(True), run(False)
    assert a._split2d is not None and a.split2d_status() == 0
    bad = _same(a, b)
    assert not bad, bad[:12]


def test_substep_kernel_in_cuda_graph():
    """Two 3D steps captured in a CUDA graph and replayed match the eager
    run bit for bit."""
    import torch

    a = _member("mixed", True, n3d=2)
    b = _member("mixed", True, n3d=2)
    n = 2 * a.split_factor
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(g, stream=stream):
            for _ in range(n):
                a.advance()
    torch.cuda.current_stream().wait_stream(stream)
    # capture ran nothing: replay the two steps, then run them eagerly on b
    g.replay()
    for _ in range(n):
        b.advance()
    torch.cuda.synchronize()
    assert a.split2d_status() == 0
    bad = _same(a, b)
    assert not bad, bad[:12]


def test_substep_error_word_leaves_state_unchanged():
    """With the error word already set (a grid barrier gave up earlier), a
    substep launch returns at once: every field and the model time stay as
    they were and the status stays non-zero, until clear_split2d_status()
    re-arms the kernel.  The error is planted on the host; no barrier times
    out."""
    import torch

    from getm_gb300 import checkpoint

    s = _member("mixed", True, n3d=1)
    assert s.split2d_status() == 0
    assert (s.istep + 1) % s.split_factor != 0  # the next advance is a one-launch substep
    before = {k: v.clone() for k, v in checkpoint.state_tensors(s).items()}
    t0 = float(s._time)
    s._split2d.sync[2] = 1
    s.advance()
    torch.cuda.synchronize()
    assert s.split2d_status() != 0
    after = checkpoint.state_tensors(s)
    changed = [k for k in before
               if not bool(((before[k] == after[k]) | (torch.isnan(before[k]) & torch.isnan(after[k]))).all())]
    assert not changed, changed[:12]
    assert float(s._time) == t0
    s.clear_split2d_status()
    assert s.split2d_status() == 0
    s.advance()
    torch.cuda.synchronize()
    assert s.split2d_status() == 0
    assert float(s._time) > t0
