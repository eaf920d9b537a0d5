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


def test_lanes_by_load():
    """A new request goes to the lane with the fewest cells of running
    requests, so small requests do not queue behind large ones."""
    from getm_gb300.serving import least_loaded

    assert least_loaded([0, 0, 0]) == 0
    assert least_loaded([5000, 100, 100]) == 1
    loads = [0] * 4
    for cells in (4000, 1000, 1000, 1000, 500, 500):
        loads[least_loaded(loads)] += cells
    assert loads == [4000, 1500, 1500, 1000]


def test_library_calls_of_a_set_up_thread_release_the_interpreter_lock():
    """An admission worker marks its thread so that every library call
    releases the interpreter lock; other threads keep the per-entry-point
    binding.  No call here launches work (the knob table is host-side)."""
    import threading

    from getm_gb300 import _lib

    seen = {}

    def worker():
        _lib.release_gil_in_this_thread()
        seen["worker"] = getattr(_lib._tls, "release", False)
        v = __import__("ctypes").c_int(0)
        _lib.call("getm_tune_get", 0, __import__("ctypes").byref(v))
        seen["value"] = v.value

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert seen["worker"] is True and seen["value"] in (2, 4, 8)
    assert getattr(_lib._tls, "release", False) is False  # this thread keeps the default


def test_no_handle_is_finalized_while_any_thread_captures():
    """Finalizing a handle frees device memory, which waits for the whole
    device: queued finalizations wait while a capture is under way on any
    thread (capture_started/ended around every capture)."""
    from getm_gb300 import _lib

    _lib.capture_started()
    try:
        assert _lib._capturing()
        _lib._pending_release.append(("getm_grid_finalize", None))
        _lib._flush_releases()
        assert _lib._pending_release  # still queued
    finally:
        _lib.capture_ended()
    assert not _lib._capturing()
    _lib._flush_releases()  # getm_grid_finalize(NULL) is a no-op
    assert not _lib._pending_release
