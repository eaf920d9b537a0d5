"""Serving loop: a request's result is the same alone and in a mix of
concurrent requests (bit for bit), admission respects the memory budget, and
every step is timed."""

import pytest

pytestmark = pytest.mark.gpu


def _requests(n, arrivals, steps=6, seed=21, precision="mixed"):
    import numpy as np

    from getm_gb300 import workloads
    from getm_gb300.serving import Request

    reqs = []
    for i in range(n):
        s = seed + i

        def make(s=s):
            return workloads.ensemble_member(np.random.default_rng(s), nmin=24, nmax=48, nzmin=5, nzmax=8)

        wl = make()
        reqs.append(Request(i, make, steps + i, arrivals[i], precision, wl.T.nx_ * wl.T.ny_ * (wl.T.nz + 1)))
    return reqs


@pytest.mark.parametrize("precision,admission_thread", [("fp64", True), ("mixed", True), ("mixed", False)])
def test_alone_equals_in_mix(precision, admission_thread):
    """Admitted on the worker thread (graphs captured while other requests'
    steps replay) or in the main loop: the same result alone and in the mix."""
    import torch

    from getm_gb300.serving import Server

    alone = Server(lanes=2, keep={0}, admission_thread=admission_thread).run(
        _requests(1, [0.0], precision=precision), duration=120.0)
    mix = Server(lanes=2, keep={0}, admission_thread=admission_thread).run(
        _requests(4, [0.0, 0.0, 0.01, 0.02], precision=precision), duration=120.0)
    a = next(r for r in alone if r.rid == 0)
    m = next(r for r in mix if r.rid == 0)
    assert a.finished and m.finished
    for name in a.final_state:
        x, y = a.final_state[name], m.final_state[name]
        same = (x == y) | (torch.isnan(x) & torch.isnan(y))
        assert bool(same.all()), name
    assert all(r.finished for r in mix)


def test_budget_and_latency():
    from getm_gb300.serving import Server, summarize

    reqs = _requests(5, [0.0] * 5)
    srv = Server(lanes=4)
    one = reqs[0]
    # calibrate the per-cell estimate, then allow about two requests at once
    Server(lanes=1).run([one], duration=60.0)
    srv.bytes_per_cell = {"mixed": 0.0}
    first = srv.run([reqs[0]], duration=60.0)
    srv.budget = 2.2 * max(srv.estimate(r) for r in reqs[1:])
    srv.used = 0.0
    srv.peak_used = 0.0
    res = srv.run(reqs[1:], duration=120.0)
    assert all(r.finished for r in first + res)
    assert srv.peak_used <= srv.budget
    s = summarize(res, 1.0)
    assert s["steps_completed"] == sum(r.nsteps for r in res)
    assert s["step_latency_p50_ms"] > 0 and s["step_latency_p99_ms"] >= s["step_latency_p50_ms"]
