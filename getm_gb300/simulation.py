"""Time-step drivers on the GPU.

``TracerTransport`` runs the tracer-transport configuration: every step is
``TracerCollection.advance`` (python/pygetm/tracer.py:193-276) - the Strang
split u/2, v/2, w, v/2, u/2 of all tracers followed by implicit vertical
diffusion - with prescribed velocities, as in python/tests/test_3d_barotropic.py.
"""

from __future__ import annotations

from typing import Optional

import torch

from .core import CENTERS, INTERFACES, Array, make_grids
from .operators import AdvectionScheme
from .tracer import TracerCollection
from .workloads import Workload


def _dev(a, device):
    return torch.from_numpy(a).to(device=device, dtype=torch.float64).contiguous()


class TracerTransport:
    """Tracer transport through prescribed (u, v, w) with vertical diffusion."""

    def __init__(self, wl: Workload, device="cuda", ntracer: int = 1):
        self.wl = wl
        self.dt = wl.params["dt"]
        self.T = T = make_grids(wl.T, device)
        for g, n in ((T, "T"), (T.ugrid, "U"), (T.vgrid, "V"), (T.xgrid, "X")):
            g.D.all_values.copy_(_dev(wl.fields[f"D_{n}"], device))
            g.hn.all_values.copy_(_dev(wl.fields[f"hn_{n}"], device))
            g.ho = Array(g, g.hn.all_values.clone(), z=CENTERS, name="ho" + g.postfix)
        T.zc.all_values.copy_(_dev(wl.fields["zc_T"], device))
        T.zf.all_values.copy_(_dev(wl.fields["zf_T"], device))
        self.uk = Array(T.ugrid, _dev(wl.fields["uk"], device), z=CENTERS, name="uk")
        self.vk = Array(T.vgrid, _dev(wl.fields["vk"], device), z=CENTERS, name="vk")
        self.w = Array(T, _dev(wl.fields["w"], device), z=INTERFACES, name="ww")
        self.nuh = Array(T, _dev(wl.fields["nuh"], device), z=INTERFACES, name="nuh")
        self.tracers = TracerCollection(T, AdvectionScheme(int(wl.params.get("scheme", 5))), cnpar=wl.params.get("cnpar", 1.0))
        c0 = _dev(wl.fields["tracer"], device)
        for t in range(ntracer):
            tr = self.tracers.add(f"tracer{t}")
            tr.all_values.copy_(c0)

    def step(self):
        self.tracers.advance(self.dt, self.uk, self.vk, self.w, self.nuh)

    def run(self, nstep: int):
        for _ in range(nstep):
            self.step()
