"""Batched ensembles of independent domains on one GPU.

Each member is a full ``Simulation`` with its own CUDA stream.  One CUDA graph
captures a period of steps of every member, each on its stream (fork from and
join back to the capture stream), so replaying the graph issues all members'
kernels with a single launch and the GPU runs the small kernels of different
members concurrently.  Members are independent: a member's results are the
same alone and in the ensemble (same kernels, same inputs, no shared state).
"""

from __future__ import annotations

from typing import List, Optional

import torch

from .simulation import Fluxes, Simulation
from .workloads import Workload


def make_member(wl: Workload, precision: str = "mixed", device="cuda") -> Simulation:
    """Build and start a simulation for one ensemble member."""
    p = wl.params
    sim = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, device=device,
                     airsea=Fluxes(taux=p.get("taux", 0.0)))
    zc = sim.T.zc.all_values
    dT = p.get("dT", 10.0)
    temp0 = torch.where(sim.T.mask.all_values[None] != 0, 20.0 + dT * zc / 100.0, sim.temp.all_values.double())
    sim.temp.all_values.copy_(temp0)
    sim.start(p["timestep"], p["split_factor"])
    return sim


class Ensemble:
    """Advance many members together through one multi-stream CUDA graph."""

    period = 2  # 3D steps per graph replay (the 3D momentum order alternates)

    def __init__(self, members: List[Simulation], device="cuda"):
        self.members = members
        self.device = torch.device(device)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in members]
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    @property
    def cells(self) -> int:
        """Interior cells of all members (the cell-update unit per 3D step)."""
        return sum(m.T.nx * m.T.ny * m.T.nz for m in self.members)

    def _advance_period(self):
        main = torch.cuda.current_stream(self.device)
        for sim, s in zip(self.members, self.streams):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                for _ in range(self.period * sim.split_factor):
                    sim.advance()
        for s in self.streams:
            main.wait_stream(s)

    def warmup(self, periods: int = 1):
        """Eager periods: allocate every work buffer before capture."""
        for _ in range(periods):
            self._advance_period()
        torch.cuda.synchronize(self.device)

    def capture(self):
        capture_stream = torch.cuda.Stream(device=self.device)
        capture_stream.wait_stream(torch.cuda.current_stream(self.device))
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(capture_stream):
            with torch.cuda.graph(self.graph, stream=capture_stream):
                self._advance_period()
        torch.cuda.current_stream(self.device).wait_stream(capture_stream)
        torch.cuda.synchronize(self.device)

    def step_period(self):
        """Advance every member by ``period`` 3D steps."""
        if self.graph is None:
            self._advance_period()
        else:
            self.graph.replay()
