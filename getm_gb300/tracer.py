"""Tracer transport on the GPU: counterpart of pygetm.tracer.TracerCollection
(python/pygetm/tracer.py:128-276) for the transport path - batched 3D
advection of all tracers followed by vertical diffusion with optional sources.
"""

from __future__ import annotations

from typing import List, Optional

import torch

from .core import CENTERS, INTERFACES, Array, Grid
from .operators import Advection, AdvectionScheme, VerticalDiffusion


class Tracer(Array):
    """A tracer field with its transport properties (python/pygetm/tracer.py:43-126)."""

    __slots__ = ("molecular_diffusivity", "source", "surface_flux", "source_scale", "vertical_velocity")

    def __init__(self, grid: Grid, name: str, molecular_diffusivity: float = 0.0, source: Optional[Array] = None,
                 surface_flux: Optional[Array] = None, source_scale: float = 1.0, fill_value=None,
                 dtype: torch.dtype = torch.float64):
        from .domain import FILL_VALUE

        data = torch.full((grid.nz, grid.ny_, grid.nx_), FILL_VALUE, dtype=dtype, device=grid.device)
        super().__init__(grid, data, z=CENTERS, fill_value=FILL_VALUE if fill_value is None else fill_value, name=name)
        self.molecular_diffusivity = molecular_diffusivity
        self.source = source
        self.surface_flux = surface_flux
        self.source_scale = source_scale
        self.vertical_velocity = None


class TracerCollection:
    """python/pygetm/tracer.py:128-276 (advance and _diffuse)."""

    def __init__(self, grid: Grid, advection_scheme: AdvectionScheme = AdvectionScheme.DEFAULT, cnpar: float = 1.0,
                 dtype: torch.dtype = torch.float64):
        """``dtype``: storage of the tracers: float64 (FP64 form, and the mixed
        form's FP64 tracer storage) or float32 (mixed form)."""
        self.grid = grid
        self.dtype = dtype
        self._tracers: List[Tracer] = []
        self._source = grid.array(z=CENTERS)
        self._advection = Advection(grid, scheme=advection_scheme)
        self._vertical_diffusion = VerticalDiffusion(grid, cnpar=cnpar)
        self._w = grid.array(fill=0.0, z=INTERFACES)
        self.Ah_u = self.Ah_v = None

    def __getitem__(self, index: int) -> Tracer:
        return self._tracers[index]

    def __len__(self) -> int:
        return len(self._tracers)

    def add(self, name: str, **kwargs) -> Tracer:
        kwargs.setdefault("dtype", self.dtype)
        t = Tracer(self.grid, name, **kwargs)
        self._tracers.append(t)
        return t

    def advance(self, timestep: float, u: Array, v: Array, w: Array, diffusivity: Array):
        """tracer.py:193-246: advection of all tracers (one fused call), then
        vertical diffusion with sources."""
        if not self._tracers:  # the reference's per-tracer loops do nothing
            return
        self._advection.apply_3d_batch(u, v, w, timestep, self._tracers, Ah_u=self.Ah_u, Ah_v=self.Ah_v)
        self._diffuse(timestep, diffusivity)

    def _diffuse(self, timestep: float, diffusivity: Array):
        """tracer.py:248-276.  prepare+apply are fused per column; each tracer
        keeps its own molecular diffusivity.  Source terms become ea4 =
        timestep * source_scale * (source + surface flux in the top layer)."""
        ea4s = []
        for tracer in self._tracers:
            if tracer.source is not None or tracer.surface_flux is not None:
                # in the solve's type (that of the diffusivity)
                src = torch.zeros_like(tracer.all_values, dtype=diffusivity.all_values.dtype)
                if tracer.source is not None:
                    src.copy_(tracer.source.all_values)
                if tracer.surface_flux is not None:
                    src[-1] += tracer.surface_flux.all_values
                src *= timestep * tracer.source_scale
                ea4s.append(Array(self.grid, src, z=CENTERS))
            else:
                ea4s.append(None)
        self._vertical_diffusion.batch(
            diffusivity, timestep, self._tracers, [t.molecular_diffusivity for t in self._tracers], None, ea4s
        )
