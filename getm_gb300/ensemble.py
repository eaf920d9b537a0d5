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

from typing import List, Optional

import torch

from .simulation import Fluxes, Simulation
from .workloads import Workload


def make_member(wl: Workload, precision: str = "mixed", device="cuda", substep_kernel: bool = False,
                concurrent_3d: bool = True) -> Simulation:
    """Build and start a simulation for one ensemble member (rest state,
    linear temperature drop ``dT`` per 100 m from 20 degC at the surface).
    Members replay concurrently on several streams, so by default their 2D
    substeps run as separate kernels rather than as one cooperative launch
    that needs every SM of the GPU at once."""
    p = wl.params
    sim = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, device=device,
                     airsea=Fluxes(taux=p.get("taux", 0.0)), substep_kernel=substep_kernel,
                     concurrent_3d=concurrent_3d)
    zc = sim.T.zc.all_values
    dT = p.get("dT", 10.0)
    temp0 = torch.where(sim.T.mask.all_values[None] != 0, 20.0 + dT * zc / 100.0, sim.temp.all_values.double())
    sim.temp.all_values.copy_(temp0)
    sim.start(p["timestep"], p["split_factor"])
    return sim


class DomainRunner:
    """Warm-up, per-step CUDA graphs and replay of one resident domain."""

    def __init__(self, sim: Simulation, warmup_steps: int = 2, use_graph: bool = True):
        self.sim = sim
        self.graphs: Optional[List[torch.cuda.CUDAGraph]] = None
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

    def prepare(self, capture_stream: Optional[torch.cuda.Stream] = None):
        """Run the eager warm-up steps (allocating every work buffer) and
        record the two step graphs.  Call on an idle device section: capture
        requires that no other thread launches work meanwhile."""
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
            with torch.cuda.stream(stream):
                with torch.cuda.graph(g, stream=stream):
                    self._eager_step()
            graphs.append(g)
        torch.cuda.current_stream(dev).wait_stream(stream)
        self.graphs = graphs

    def step(self):
        """Issue one 3D step on the current stream."""
        if self.graphs is None:
            self._eager_step()
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
