"""Host-side accounting of the serving leg (getm_gb300.serving.summarize):
per-step latencies from the device timestamps of each request's steps,
finished requests, throughput over the span from the first admission to the
last completed step, and the admission wait."""

import numpy as np
import pytest


def test_summarize_latencies_throughput_and_waits():
    from getm_gb300.serving import Result, summarize

    a = Result(rid=0, cells=1000, nsteps=3, arrival=0.0, admitted=0.5, step_done=[1.0, 1.1, 1.3])
    b = Result(rid=1, cells=4000, nsteps=4, arrival=0.2, admitted=1.2, step_done=[1.5, 2.0])
    s = summarize([a, b], wall=3.0)
    assert s["requests_admitted"] == 2
    assert s["requests_finished"] == 1  # b completed 2 of its 4 steps
    assert s["steps_completed"] == 5
    deltas = np.array([0.1, 0.2, 0.5])
    assert s["step_latency_p50_ms"] == pytest.approx(np.percentile(deltas, 50) * 1e3)
    assert s["step_latency_p99_ms"] == pytest.approx(np.percentile(deltas, 99) * 1e3)
    # 1000 cells x 3 steps + 4000 x 2 over 0.5 s .. 2.0 s
    assert s["cell_updates_per_s"] == pytest.approx((3000 + 8000) / 1.5)
    assert s["admission_wait_p50_s"] == pytest.approx(np.median([0.5, 1.0]))
    assert s["wall_s"] == 3.0


def test_summarize_without_completed_steps():
    from getm_gb300.serving import Result, summarize

    s = summarize([Result(rid=0, cells=10, nsteps=2, arrival=0.0, admitted=0.1)], wall=1.0)
    assert s["steps_completed"] == 0 and s["requests_finished"] == 0
    assert s["step_latency_p50_ms"] is None and s["step_latency_p99_ms"] is None
    assert summarize([], wall=1.0)["admission_wait_p50_s"] is None
