"""Serving loop: continuous batching of simulation requests on one GPU.

A request is a domain plus a number of 3D steps.  Requests arrive over time;
one is admitted as soon as its estimated device memory fits the HBM budget
(first come, first served), built, warmed up and recorded into step graphs
(``ensemble.DomainRunner``), and from then on advanced one 3D step at a time
by graph replay on one of a few lane streams, interleaved with every other
active request, so requests that arrive while others run join the mix and
their work overlaps on the device.  A finished request leaves the mix; its
memory returns to the budget when no request is running (releasing a
domain's library buffers waits for all work on the device, so it is not
done while other requests' steps are queued).  Its state stays resident in
HBM for its whole life.

Admission runs on a worker thread with its own stream: building a domain,
its eager warm-up steps and the capture of its step graphs (in thread-local
capture mode) overlap with the main loop, which only decides admissions,
issues graph replays and polls completions, so issuing the steps of running
requests never waits for a request being set up.  Replays go through the
library's getm_graph_launch on lane streams the server creates for itself
(never torch's pooled streams, one of which a capture may have drawn in),
and the worker's library calls release the interpreter lock.  Kernels should
be loaded when the CUDA context is created (CUDA_MODULE_LOADING=EAGER set
before CUDA starts): loading one at its first launch on a busy device holds
up every thread's CUDA calls.

Every step's completion is timed on the device (a CUDA event per step,
measured against a start event), which gives the per-step latency: the time
between consecutive completed 3D steps of a request.
"""

from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np
import torch

from . import _lib
from .ensemble import RAW_LAUNCH, DomainRunner, make_member
from .workloads import Workload

GB = 1e9


@dataclass
class Request:
    rid: int
    make_workload: Callable[[], Workload]  # built at admission
    nsteps: int
    arrival: float                         # seconds after the start of the run
    precision: str = "mixed"
    cells_hint: int = 0                    # nx * ny * (nz + 1), for the memory estimate


@dataclass
class Result:
    rid: int
    cells: int
    nsteps: int
    arrival: float
    admitted: float = float("nan")
    step_done: List[float] = field(default_factory=list)  # device time of each completed step (s)
    final_state: Optional[Dict[str, torch.Tensor]] = None

    @property
    def finished(self) -> bool:
        return len(self.step_done) >= self.nsteps


class _Active:
    def __init__(self, req: Request, runner: DomainRunner, estimate: float, lane: torch.cuda.Stream):
        self.req = req
        self.runner = runner
        self.estimate = estimate
        self.lane = lane
        self.inflight: List[torch.cuda.Event] = []


def least_loaded(loads: List[int]) -> int:
    """Index of the lane with the fewest cells of running requests (the
    first such lane on a tie)."""
    return min(range(len(loads)), key=lambda k: loads[k])


class Server:
    """Continuous-batching server for one GPU.

    ``budget_bytes``: device memory the resident requests may use (estimated
    per request from its cell count, calibrated on the first admissions).
    ``lanes``: streams the active requests are spread over.
    ``max_inflight``: steps a request may have queued on the device at once.
    ``keep``: request ids whose final state is copied out for inspection.
    """

    STATE_FIELDS = ("temp", "salt")

    def __init__(self, budget_bytes: float = 150 * GB, lanes: int = 32, max_inflight: int = 2,
                 device="cuda", keep=(), admission_thread: bool = True, max_building: int = 2):
        """``admission_thread``: set requests up on a worker thread (False:
        in the main loop, between step issues); ``max_building``: requests
        handed to the worker and not yet ready."""
        self.device = torch.device(device)
        self.budget = float(budget_bytes)
        # lanes of the caller's own (torch's pooled streams can coincide with
        # a stream that a set-up capture draws in, and a launch into a
        # capturing stream fails)
        self.lanes = [_lib.own_stream(self.device) for _ in range(lanes)]
        self.max_inflight = max_inflight
        self.keep = set(keep)
        self.bytes_per_cell: Dict[str, float] = {}
        self.default_bytes_per_cell = 2000.0
        self.used = 0.0
        self.peak_used = 0.0
        # set-up work (eager warm-up steps) on high-priority streams: its
        # kernels go ahead of the queued step replays of running requests
        self._capture_stream = _lib.own_stream(self.device, priority=-1)
        self._build_stream = _lib.own_stream(self.device, priority=-1)
        self._lane_cells = [0] * lanes
        self._lane_mutex = threading.Lock()
        # held by the admission worker while it captures a graph and by the
        # main loop while it issues replays, where those go through torch's
        # CUDAGraph.replay (which refuses a replay while any graph is being
        # captured); replays through getm_graph_launch need no lock
        self._capture_lock = threading.Lock()
        self._lock_replays = not RAW_LAUNCH
        self.admission_thread = admission_thread
        self.max_building = max(1, max_building)
        self.admission_host_s: List[float] = []

    def estimate(self, req: Request) -> float:
        bpc = self.bytes_per_cell.get(req.precision, self.default_bytes_per_cell)
        return 1.1 * bpc * max(req.cells_hint, 1)

    @staticmethod
    def resident_bytes(sim) -> int:
        """Device bytes of a simulation's fields (every state tensor once)."""
        from .checkpoint import state_tensors

        seen, total = set(), 0
        for t in state_tensors(sim).values():
            s = t.untyped_storage()
            if t.device.type != "cuda" or s.data_ptr() in seen:
                continue
            seen.add(s.data_ptr())
            total += s.nbytes()
        return total

    def _admit(self, req: Request, wl: Workload, t_run: float, start: torch.cuda.Event,
               capture_error_mode: str = "global") -> _Active:
        sim = make_member(wl, req.precision, device=self.device)
        runner = DomainRunner(sim)
        res = Result(req.rid, runner.cells, req.nsteps, req.arrival, admitted=t_run)
        # warm-up steps run eagerly inside prepare(); time them as one block
        runner.prepare(self._capture_stream, capture_error_mode,
                       capture_lock=self._capture_lock if capture_error_mode == "thread_local" else None)
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        ev.synchronize()
        t_done = start.elapsed_time(ev) / 1000.0
        res.step_done.extend([t_done] * min(runner.steps_done, req.nsteps))
        # fields plus operator work buffers and graph pools (about a third more)
        grown = 1.35 * self.resident_bytes(sim)
        cells = wl.T.nx_ * wl.T.ny_ * (wl.T.nz + 1)
        bpc = grown / cells
        self.bytes_per_cell[req.precision] = max(self.bytes_per_cell.get(req.precision, 0.0), bpc)
        # the lane with the fewest cells of running requests (a lane runs its
        # requests' steps one after another)
        with self._lane_mutex:
            li = least_loaded(self._lane_cells)
            self._lane_cells[li] += runner.cells
        a = _Active(req, runner, max(self.estimate(req), 1.05 * grown), self.lanes[li])
        a.lane_index = li
        a.result = res
        return a

    def _worker(self, inbox: "queue.Queue", ready: "queue.Queue", start: torch.cuda.Event, t0: float):
        """Admission worker: build, warm up and capture each handed request
        on the worker's own stream; hand the result (or the exception) back.
        Its library calls release the interpreter lock (one that blocks must
        not stop the main loop's step issue)."""
        _lib.release_gil_in_this_thread()
        while True:
            item = inbox.get()
            if item is None:
                return
            req, fut, t_adm = item
            try:
                wl = fut.result() if fut is not None else req.make_workload()
                ta = time.perf_counter()
                with torch.cuda.stream(self._build_stream):
                    a = self._admit(req, wl, t_adm, start, capture_error_mode="thread_local")
                self.admission_host_s.append(time.perf_counter() - ta)
                ready.put(a)
            except BaseException as e:  # surfaced by the main loop
                ready.put(e)

    def run(self, requests: List[Request], duration: float, admit_until: Optional[float] = None,
            poll_sleep: Optional[float] = None) -> List[Result]:
        """Serve ``requests`` until all admitted ones are done or ``duration``
        seconds have passed (unfinished work is then abandoned; its completed
        steps still count).  Requests are admitted until ``admit_until``
        seconds (default: ``duration``).  Workloads of the next arrivals are
        generated on a host thread ahead of their admission; with
        ``admission_thread`` the set-up runs on a worker thread, otherwise at
        most one request is set up per pass of the loop.  ``poll_sleep``:
        seconds the loop sleeps when a pass found nothing to do, doubled
        after each idle pass up to 8 times that, reset when a step completes
        or is issued (default: 0.5 ms with the admission thread, which then
        gets the interpreter: a loop that polls every 100 us held it half the
        time and slowed the worker's set-up tenfold; every request keeps
        max_inflight steps queued, milliseconds of device work; 0 without).
        Returns one Result per admitted request."""
        import queue
        import sys
        import threading
        from concurrent.futures import ThreadPoolExecutor

        admit_until = duration if admit_until is None else admit_until
        if poll_sleep is None:
            poll_sleep = 5e-4 if self.admission_thread else 0.0
        idle_sleep = poll_sleep
        pending = sorted(requests, key=lambda r: r.arrival)
        active: List[_Active] = []
        results: List[Result] = []
        prefetch = ThreadPoolExecutor(max_workers=1)  # one host thread keeps ahead of admission
        futures: Dict[int, object] = {}

        def prefetch_ahead():
            for r in pending[:4]:
                if r.rid not in futures:
                    futures[r.rid] = prefetch.submit(r.make_workload)

        start = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(self.device)
        start.record()
        t0 = time.perf_counter()
        self.admission_host_s = []
        self._lane_cells = [0] * len(self.lanes)
        inbox: "queue.Queue" = queue.Queue()
        ready: "queue.Queue" = queue.Queue()
        reserved: Dict[int, float] = {}
        worker = None
        switch = sys.getswitchinterval()
        if self.admission_thread:
            # the main loop's short bursts of step issue should not wait a
            # whole default switch interval behind the worker's set-up
            sys.setswitchinterval(5e-4)
            worker = threading.Thread(target=self._worker, args=(inbox, ready, start, t0), daemon=True)
            worker.start()

        retired: List[_Active] = []

        def release_retired():
            for a in retired:
                self.used -= a.estimate
                a.runner = None
            retired.clear()

        def take(a: _Active):
            self.used += a.estimate - reserved.pop(a.req.rid, 0.0)
            self.peak_used = max(self.peak_used, self.used)
            active.append(a)
            results.append(a.result)

        try:
            while True:
                now = time.perf_counter() - t0
                if now > duration:
                    break
                prefetch_ahead()
                # requests the worker finished setting up join the mix
                while not ready.empty():
                    a = ready.get_nowait()
                    if isinstance(a, BaseException):
                        raise a
                    take(a)
                # admission: first come, first served, while the budget allows
                if pending and pending[0].arrival <= now and now <= admit_until and len(reserved) < (
                        self.max_building if worker is not None else 1):
                    est = self.estimate(pending[0])
                    if self.used + est <= self.budget or (not active and not reserved):
                        req = pending.pop(0)
                        fut = futures.pop(req.rid, None)
                        reserved[req.rid] = est
                        self.used += est
                        self.peak_used = max(self.peak_used, self.used)
                        if worker is not None:
                            inbox.put((req, fut, now))
                        else:
                            wl = fut.result() if fut is not None else req.make_workload()
                            ta = time.perf_counter()
                            a = self._admit(req, wl, ta - t0, start)
                            self.admission_host_s.append(time.perf_counter() - ta)
                            take(a)
                # completion of issued steps, then issue the next ones (not
                # while the worker captures a graph: this pass skips them)
                progressed = False
                may_issue = self._capture_lock.acquire(blocking=False) if self._lock_replays else True
                try:
                    for a in active:
                        while a.inflight and a.inflight[0].query():
                            ev = a.inflight.pop(0)
                            a.result.step_done.append(start.elapsed_time(ev) / 1000.0)
                            progressed = True
                        issued = len(a.result.step_done) + len(a.inflight)
                        while may_issue and issued < a.req.nsteps and len(a.inflight) < self.max_inflight:
                            with torch.cuda.stream(a.lane):
                                a.runner.step()
                                ev = torch.cuda.Event(enable_timing=True)
                                ev.record(a.lane)
                            a.inflight.append(ev)
                            issued += 1
                            progressed = True
                finally:
                    if may_issue and self._lock_replays:
                        self._capture_lock.release()
                # retire finished requests
                keep_active = []
                for a in active:
                    if a.result.finished and not a.inflight:
                        if a.req.rid in self.keep:
                            sim = a.runner.sim
                            a.result.final_state = {n: getattr(sim, n).all_values.clone() for n in self.STATE_FIELDS}
                            a.result.final_state["z"] = sim.T.z.all_values.clone()
                            a.result.final_state["U"] = sim.momentum.U.all_values.clone()
                        # released later, with the device idle: freeing a
                        # domain's library buffers (cudaFree) waits for all
                        # work on the device, every other request's queued
                        # steps included
                        retired.append(a)
                        with self._lane_mutex:
                            self._lane_cells[a.lane_index] -= a.runner.cells
                    else:
                        keep_active.append(a)
                active = keep_active
                if retired and not active and not reserved:
                    release_retired()
                if not active and not reserved and (not pending or now > admit_until):
                    break
                if progressed:
                    idle_sleep = poll_sleep
                elif poll_sleep > 0:
                    # back off while nothing completes (a pass that wakes every
                    # 100 us would hold the interpreter half the time and
                    # starve the admission worker); every request keeps
                    # max_inflight steps queued, so the device does not wait
                    time.sleep(idle_sleep)
                    idle_sleep = min(2.0 * idle_sleep, 8.0 * poll_sleep)
        finally:
            if worker is not None:
                inbox.put(None)
                worker.join()
                sys.setswitchinterval(switch)
                while not ready.empty():  # set up but never joined the mix
                    a = ready.get_nowait()
                    if not isinstance(a, BaseException):
                        a.runner = None
            prefetch.shutdown(wait=True, cancel_futures=True)
        torch.cuda.synchronize(self.device)
        release_retired()
        for a in active:  # abandoned at the deadline: count what completed
            for ev in a.inflight:
                a.result.step_done.append(start.elapsed_time(ev) / 1000.0)
            a.runner = None
        return results


def summarize(results: List[Result], wall: float) -> dict:
    """Per-step latency percentiles and aggregate throughput of a run."""
    deltas = []
    cell_updates = 0
    first, last = float("inf"), 0.0
    for r in results:
        t = r.step_done
        cell_updates += r.cells * len(t)
        deltas.extend(np.diff(np.asarray(t)).tolist())
        if t:
            first = min(first, r.admitted)
            last = max(last, t[-1])
    d = np.asarray([x for x in deltas if x > 0.0])
    span = max(last - (first if first < float("inf") else 0.0), 1e-9)
    return {
        "requests_admitted": len(results),
        "requests_finished": sum(r.finished for r in results),
        "steps_completed": int(sum(len(r.step_done) for r in results)),
        "step_latency_p50_ms": float(np.percentile(d, 50) * 1e3) if d.size else None,
        "step_latency_p99_ms": float(np.percentile(d, 99) * 1e3) if d.size else None,
        "cell_updates_per_s": cell_updates / span,
        "wall_s": wall,
        "admission_wait_p50_s": float(np.median([r.admitted - r.arrival for r in results])) if results else None,
    }
