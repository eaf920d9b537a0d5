"""The 3D step on two streams (Simulation(concurrent_3d=True)): the advection
of the 3D momentum and the slow terms run beside the tracers, density and
internal pressure.  The state is bit for bit that of the one-stream step, in
both forms, eagerly and replayed from CUDA graphs."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    import torch

    from getm_gb300 import checkpoint

    sa, sb = checkpoint.state_tensors(a), checkpoint.state_tensors(b)
    return [k for k in sa if not bool(((sa[k] == sb[k]) | (torch.isnan(sa[k]) & torch.isnan(sb[k]))).all())]


def _member(precision, concurrent, substep_kernel=True, seed=5):
    from getm_gb300 import workloads
    from getm_gb300.ensemble import make_member

    wl = workloads.ensemble_member(np.random.default_rng(seed), nmin=40, nmax=48, nzmin=6, nzmax=8)
    s = make_member(wl, precision, substep_kernel=substep_kernel, concurrent_3d=concurrent)
    assert (s._side_stream is not None) == concurrent
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_concurrent_3d_is_bitwise(precision):
    import torch

    a, b = _member(precision, True), _member(precision, False)
    for s in (a, b):
        for _ in range(4 * s.split_factor):
            s.advance()
    torch.cuda.synchronize()
    assert not _same(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_concurrent_3d_graph_replay_is_bitwise(precision):
    """Two-stream steps captured into CUDA graphs (the side stream joins the
    capture and rejoins it before the next substep) against eager
    one-stream steps."""
    import torch

    from getm_gb300.ensemble import DomainRunner

    a, b = _member(precision, True), _member(precision, False)
    r = DomainRunner(a, warmup_steps=2, use_graph=True)
    r.prepare()
    for _ in range(3):
        r.step()
    torch.cuda.synchronize()
    for _ in range(r.steps_done * b.split_factor):
        b.advance()
    torch.cuda.synchronize()
    assert r.graphs is not None
    assert not _same(a, b)
