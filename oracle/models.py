"""Oracle time-step drivers (numpy + C restatement) - TEST INFRASTRUCTURE ONLY.

``TracerTransport`` restates TracerCollection.advance / _diffuse
(python/pygetm/tracer.py:193-276) on the oracle operators, started from the
same ``Workload`` arrays as the GPU driver.
"""

from __future__ import annotations

import numpy as np

from . import oracle as O


class TracerTransport:
    def __init__(self, wl, ntracer: int = 1):
        self.wl = wl
        self.dt = wl.params["dt"]
        self.T = T = O.make_grids(wl.T)
        for g, n in ((T, "T"), (T.ugrid, "U"), (T.vgrid, "V"), (T.xgrid, "X")):
            g.D[...] = wl.fields[f"D_{n}"]
            g.hn[...] = wl.fields[f"hn_{n}"]
            g.ho[...] = g.hn
        T.zc[...] = wl.fields["zc_T"]
        T.zf[...] = wl.fields["zf_T"]
        self.uk = np.ascontiguousarray(wl.fields["uk"])
        self.vk = np.ascontiguousarray(wl.fields["vk"])
        self.w = np.ascontiguousarray(wl.fields["w"])
        self.nuh = np.ascontiguousarray(wl.fields["nuh"])
        self.adv = O.Advection(T, O.AdvectionScheme(int(wl.params.get("scheme", 5))))
        self.vdif = O.VerticalDiffusion(T, cnpar=wl.params.get("cnpar", 1.0))
        self.tracers = [np.ascontiguousarray(wl.fields["tracer"]).copy() for _ in range(ntracer)]
        self.molecular = [0.0] * ntracer

    def step(self):
        self.adv.apply_3d_batch(self.uk, self.vk, self.w, self.dt, self.tracers)
        avmol = -1.0
        for tracer, mol in zip(self.tracers, self.molecular):
            if mol != avmol:
                avmol = mol
                self.vdif.prepare(self.nuh, self.dt, avmol)
            self.vdif.apply(tracer)

    def run(self, nstep: int):
        for _ in range(nstep):
            self.step()
