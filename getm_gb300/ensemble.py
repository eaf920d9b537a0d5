"""Batched ensembles of independent domains on one GPU.

Each member is a full ``Simulation`` whose state stays resident in HBM.  A
``DomainRunner`` records the member's 3D steps into CUDA graphs after a short
eager warm-up: two graphs, one per parity of the 3D step (the 3D momentum
update alternates its u/v order every step and the 2D one every substep), so
a replay advances the member by exactly one 3D step with a single launch.
``Ensemble`` replays every member's graph on one of a few "lane" streams, so
the small kernels of different members run concurrently on the GPU; members
share no state, so a member's results are the same alone and in the ensemble.
"""

from __future__ import annotations

import contextlib

from typing import List, Optional

import torch

from . import _lib
from .simulation import Fluxes, Simulation
from .workloads import Workload


def make_member(wl: Workload, precision: str = "mixed", device="cuda", substep_kernel: bool = False,
                concurrent_3d: bool = True, tiles=None) -> Simulation:
    """Build and start a simulation for one ensemble member (rest state,
    linear temperature drop ``dT`` per 100 m from 20 degC at the surface).
    Members replay concurrently on several streams, so by default their 2D
    substeps run as separate kernels rather than as one cooperative launch
    that needs every SM of the GPU at once.  ``tiles``: launch shapes
    (``Simulation``), e.g. "auto" for the tuned shapes of the member's size."""
    p = wl.params
    sim = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, device=device,
                     airsea=Fluxes(taux=p.get("taux", 0.0)), substep_kernel=substep_kernel,
                     concurrent_3d=concurrent_3d, tiles=tiles)
    zc = sim.T.zc.all_values
    dT = p.get("dT", 10.0)
    temp0 = torch.where(sim.T.mask.all_values[None] != 0, 20.0 + dT * zc / 100.0, sim.temp.all_values.double())
    sim.temp.all_values.copy_(temp0)
    sim.start(p["timestep"], p["split_factor"])
    return sim


# PyTorch exposes the instantiated graph (cudaGraphExec_t): replays then go
# through the library's getm_graph_launch, which another host thread may
# call while one captures (torch's CUDAGraph.replay refuses that)
RAW_LAUNCH = hasattr(torch.cuda.CUDAGraph, "raw_cuda_graph_exec")


class DomainRunner:
    """Warm-up, per-step CUDA graphs and replay of one resident domain."""

    def __init__(self, sim: Simulation, warmup_steps: int = 2, use_graph: bool = True):
        self.sim = sim
        self.graphs: Optional[List[torch.cuda.CUDAGraph]] = None
        self._execs: Optional[List[int]] = None  # the graphs' cudaGraphExec_t (RAW_LAUNCH)
        self.steps_done = 0  # 3D steps completed on the device (as issued)
        self._use_graph = use_graph
        self._warmup = warmup_steps + warmup_steps % 2

    @property
    def cells(self) -> int:
        T = self.sim.T
        return T.nx * T.ny * T.nz

    def _eager_step(self):
        for _ in range(self.sim.split_factor):
            self.sim.advance()

    def prepare(self, capture_stream: Optional[torch.cuda.Stream] = None, capture_error_mode: str = "global",
                capture_lock=None):
        """Run the eager warm-up steps (allocating every work buffer) and
        record the two step graphs.  ``capture_error_mode="thread_local"``
        lets other host threads keep launching work (event queries, kernels)
        while this one captures; with "global" no other thread may make CUDA
        calls during the capture.  ``capture_lock``: held during each
        capture; another thread that replays graphs must hold it too (torch
        refuses a replay while any graph is being captured)."""
        for _ in range(self._warmup):
            self._eager_step()
        self.steps_done = self._warmup
        if not self._use_graph:
            return
        dev = self.sim.T.device
        stream = capture_stream or torch.cuda.Stream(device=dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        graphs = []
        for _ in range(2):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(stream), (capture_lock or contextlib.nullcontext()):
                # capture_begin/end rather than the torch.cuda.graph context,
                # which synchronizes the whole device, collects garbage and
                # empties the allocator's cache first: with other domains'
                # steps queued (serving) that waits for all of them
                _lib.capture_started()
                try:
                    g.capture_begin(capture_error_mode=capture_error_mode)
                    try:
                        self._eager_step()
                    finally:
                        g.capture_end()
                finally:
                    _lib.capture_ended()
            graphs.append(g)
        torch.cuda.current_stream(dev).wait_stream(stream)
        self.graphs = graphs
        if RAW_LAUNCH:
            self._execs = [int(g.raw_cuda_graph_exec()) for g in graphs]

    def step(self):
        """Issue one 3D step on the current stream."""
        if self.graphs is None:
            self._eager_step()
        elif self._execs is not None:
            dev = self.sim.T.device
            try:
                _lib.graph_launch(self._execs[(self.steps_done - self._warmup) % 2],
                                  torch.cuda.current_stream(dev).cuda_stream)
            except _lib.GetmError as e:
                # name the device's error, if it holds one
                try:
                    torch.cuda.current_stream(dev).synchronize()
                except RuntimeError as d:
                    raise RuntimeError(f"{e}; the stream reports: {d}") from e
                raise
        else:
            self.graphs[(self.steps_done - self._warmup) % 2].replay()
        self.steps_done += 1


class Ensemble:
    """Advance many members together: each member's step graph is replayed on
    one of ``lanes`` streams (round robin), one 3D step per member per call."""

    def __init__(self, members: List[Simulation], lanes: int = 16, use_graph: bool = True, device="cuda"):
        self.device = torch.device(device)
        self.runners = [DomainRunner(m, use_graph=use_graph) for m in members]
        self.lanes = [torch.cuda.Stream(device=self.device) for _ in range(max(1, min(lanes, len(members))))]

    @property
    def members(self) -> List[Simulation]:
        return [r.sim for r in self.runners]

    @property
    def cells(self) -> int:
        """Interior cells of all members (the cell-update unit per 3D step)."""
        return sum(r.cells for r in self.runners)

    def prepare(self):
        capture_stream = torch.cuda.Stream(device=self.device)
        for r in self.runners:
            r.prepare(capture_stream)
        torch.cuda.synchronize(self.device)

    def step(self, sequential: bool = False, events: Optional[List[torch.cuda.Event]] = None):
        """One 3D step of every member.  ``sequential``: all members on the
        current stream, one after the other (the single-domain reference).
        ``events``: one event per member, recorded after its step."""
        main = torch.cuda.current_stream(self.device)
        if sequential:
            for n, r in enumerate(self.runners):
                r.step()
                if events is not None:
                    events[n].record(main)
            return
        for s in self.lanes:
            s.wait_stream(main)
        for n, r in enumerate(self.runners):
            s = self.lanes[n % len(self.lanes)]
            with torch.cuda.stream(s):
                r.step()
                if events is not None:
                    events[n].record(s)
        for s in self.lanes:
            main.wait_stream(s)


class BatchedEnsemble:
    """Advance many members together with the 2D substeps of all members in
    one persistent kernel: per 3D step (a "round"), one cooperative launch
    per substep index k advances every member with more than k substeps left
    before its 3D step (``getm_substep_batch_launch``), then every member's
    last substep and its 3D step run on one of ``lanes`` streams.  Members
    may differ in size and in their number of substeps.  Each round is
    replayed from CUDA graphs: one graph of the batched launches per parity
    of the round, and one graph of each member's 3D substep per parity.

    Members must be built with ``substep_kernel=True`` (each then carries the
    fields of the one-launch substep) and share one precision form; their
    results are bitwise those of advancing each alone."""

    def __init__(self, members: List[Simulation], lanes: int = 16, warmup_rounds: int = 2, device="cuda"):
        import ctypes

        from ._lib import call

        self.device = torch.device(device)
        self.members = list(members)
        if not self.members:
            raise ValueError("empty ensemble")
        forms = {m.precision for m in self.members}
        if len(forms) != 1:
            raise ValueError(f"members of one precision form only, not {sorted(forms)}")
        for m in self.members:
            if m._split2d is None:
                raise ValueError("every member needs the one-launch substep (substep_kernel=True and a "
                                 "configuration it covers)")
        self.mixed = forms.pop() == "mixed"
        self.lanes = [torch.cuda.Stream(device=self.device) for _ in range(max(1, min(lanes, len(self.members))))]
        self.sync = torch.zeros(4, dtype=torch.int32, device=self.device)
        h = ctypes.c_void_p()
        call("getm_substep_batch_create", len(self.members), int(self.mixed), ctypes.byref(h))
        self._h = h
        self._warmup = warmup_rounds + warmup_rounds % 2
        self.rounds_done = 0
        self.graphs = None
        self.nsub = [m.split_factor - 1 for m in self.members]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            from ._lib import release

            try:
                release("getm_substep_batch_finalize", h)
            except Exception:
                pass

    @property
    def cells(self) -> int:
        return sum(m.T.nx * m.T.ny * m.T.nz for m in self.members)

    def status(self) -> int:
        """Non-zero when a grid barrier of the batched substep gave up."""
        return int(self.sync[2].item())

    def _register(self):
        """The members' fields and orders at the start of an even round."""
        import ctypes

        from ._lib import call

        for q, s in enumerate(self.members):
            T, U, V, m = s.T, s.U, s.V, s.momentum
            call("getm_substep_batch_set", self._h, q, self.nsub[q], s.split_factor, ctypes.byref(s._split2d.fields),
                 T.nx_, T.ny_, T.halox, T.haloy, int(bool(m._ufirst)), 1, int(bool(m.apply_bottom_friction)),
                 float(s.timestep), float(s.Dmin), float(s.Dcrit),
                 m.uadv.p, U.handle, U.ugrid.handle, U.vgrid.handle, int(m.uadv.ufirst),
                 m.vadv.p, V.handle, V.ugrid.handle, V.vgrid.handle, int(m.vadv.ufirst))
        call("getm_substep_batch_upload", self._h)

    def _batched_substeps(self, round_parity: int):
        """The launches of one round, with the members' host-side counters
        moved on as advance() would."""
        from ._lib import call

        for k in range(max(self.nsub)):
            call("getm_substep_batch_launch", self._h, k, round_parity, self.sync.data_ptr(),
                 torch.cuda.current_stream(self.device).cuda_stream)
        for s, n in zip(self.members, self.nsub):
            s.istep += n
            if n % 2:
                s.momentum._ufirst = not s.momentum._ufirst

    def _macro(self, main, events=None):
        """Every member's last substep (with its 3D step) on the lanes."""
        for st in self.lanes:
            st.wait_stream(main)
        for q, s in enumerate(self.members):
            st = self.lanes[q % len(self.lanes)]
            with torch.cuda.stream(st):
                s.advance()
                if events is not None:
                    events[q].record(st)
        for st in self.lanes:
            main.wait_stream(st)

    def prepare(self):
        """Warm-up rounds member by member (allocating every work buffer),
        the device table, and the round graphs (one per round parity)."""
        for s in self.members:
            for _ in range(self._warmup * s.split_factor):
                s.advance()
        torch.cuda.synchronize(self.device)
        self._register()
        self.rounds_done = 0
        main = torch.cuda.Stream(device=self.device)
        main.wait_stream(torch.cuda.current_stream(self.device))
        self.graphs = []
        with torch.cuda.stream(main):
            for r in range(2):
                gb = torch.cuda.CUDAGraph()
                with torch.cuda.graph(gb, stream=main):
                    self._batched_substeps(r)
                gm = []
                for s in self.members:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=main):
                        s.advance()
                    gm.append(g)
                self.graphs.append((gb, gm))
        torch.cuda.current_stream(self.device).wait_stream(main)
        torch.cuda.synchronize(self.device)

    def step(self, events: Optional[List[torch.cuda.Event]] = None):
        """One round: every member advances by one 3D step.  ``events``: one
        per member, recorded after its 3D step."""
        main = torch.cuda.current_stream(self.device)
        if self.graphs is None:
            self._batched_substeps(self.rounds_done % 2)
            self._macro(main, events)
        else:
            gb, gm = self.graphs[self.rounds_done % 2]
            gb.replay()
            for st in self.lanes:
                st.wait_stream(main)
            for q, g in enumerate(gm):
                st = self.lanes[q % len(self.lanes)]
                with torch.cuda.stream(st):
                    g.replay()
                    if events is not None:
                        events[q].record(st)
            for st in self.lanes:
                main.wait_stream(st)
        self.rounds_done += 1
