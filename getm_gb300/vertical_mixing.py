"""Vertical mixing: counterpart of pygetm.vertical_mixing
(python/pygetm/vertical_mixing.py:14-188).

``VerticalMixing`` provides prescribed turbulent viscosity ``num`` and
diffusivity ``nuh`` (zero unless set), as the reference's base class does.
``GOTM`` computes them with a two-equation closure each 3D step.  The
reference calls the external GOTM library there; this class runs the
library's own k-epsilon kernel instead (``getm_keps_advance``: the
buoyancy-extended k-epsilon model of Rodi 1987 with constant stability
functions, log-law boundary values and the Galperin length-scale limit),
keeping the reference's interface (``initialize``, ``advance`` with ustar_s,
ustar_b, z0s, z0b, NN, SS; state ``tke``, ``eps``, ``L``, ``num``, ``nuh``).
"""

from __future__ import annotations

import ctypes
from typing import Optional

import torch

from .core import INTERFACES, Array, Grid
from .domain import FILL_VALUE


class VerticalMixing:
    """python/pygetm/vertical_mixing.py:14-57: prescribed num and nuh."""

    _ob = None  # the simulation's open boundaries (DeviceBoundaries), if any

    def initialize(self, grid: Grid, dtype: torch.dtype = torch.float64):
        self.grid = grid
        self.nuh = grid.array(z=INTERFACES, name="nuh", dtype=dtype)
        self.num = grid.array(z=INTERFACES, name="num", dtype=dtype)
        self.nuh.fill(0.0)
        self.num.fill(0.0)

    def advance(self, timestep: float, ustar_s: Array, ustar_b: Array, z0s: Array, z0b: Array, NN: Array,
                SS: Array):
        pass


class KEpsParams(ctypes.Structure):
    """getm_keps_params (include/getm_gb300.h)."""

    _fields_ = [(n, ctypes.c_double) for n in
                ("cm0", "kappa", "sig_k", "sig_e", "c1", "c2", "c3_minus", "c3_plus", "galp", "prandtl", "k_min",
                 "eps_min")]


class GOTM(VerticalMixing):
    """python/pygetm/vertical_mixing.py:60-188 with the library's k-epsilon
    closure.  ``params``: overrides of the model constants (names of
    ``KEpsParams``).  tke, eps and L are FP64; num and nuh have the
    simulation's 3D type."""

    def __init__(self, path: Optional[str] = None, params: Optional[dict] = None):
        super().__init__()
        if path is not None:
            raise NotImplementedError("GOTM namelist/YAML configuration files are not read; pass params")
        self.params = KEpsParams()
        from ._lib import call

        call("getm_keps_default_params", ctypes.addressof(self.params))
        for k, v in (params or {}).items():
            if not hasattr(self.params, k):
                raise KeyError(f"unknown k-epsilon parameter {k!r}")
            setattr(self.params, k, float(v))

    def initialize(self, grid: Grid, dtype: torch.dtype = torch.float64):
        super().initialize(grid, dtype)
        p = self.params
        cde = p.cm0 * p.cm0 * p.cm0
        cmu = p.cm0 * p.cm0 * p.cm0 * p.cm0
        self.tke = grid.array(z=INTERFACES, name="tke", fill_value=FILL_VALUE)
        self.eps = grid.array(z=INTERFACES, name="eps", fill_value=FILL_VALUE)
        self.L = grid.array(z=INTERFACES, name="L", fill_value=FILL_VALUE)
        # the initial turbulence of a GOTM start: k = k_min, eps = eps_min
        self.tke.fill(p.k_min)
        self.eps.fill(p.eps_min)
        self.L.fill(cde * p.k_min * p.k_min ** 0.5 / p.eps_min)
        nu = cmu * p.k_min * p.k_min / p.eps_min
        self.num.fill(nu)
        self.nuh.fill(nu / p.prandtl)
        self._work = torch.empty(2 * (grid.nz + 1) * grid.ny_ * grid.nx_, dtype=torch.float64, device=grid.device)

    def advance(self, timestep: float, ustar_s: Array, ustar_b: Array, z0s: Array, z0b: Array, NN: Array,
                SS: Array):
        """vertical_mixing.py:136-188"""
        from ._lib import call
        from .core import _sfx

        g = self.grid
        assert ustar_s.grid is g and ustar_s.ndim == 2
        assert ustar_b.grid is g and ustar_b.ndim == 2
        assert z0s.grid is g and z0s.ndim == 2
        assert z0b.grid is g and z0b.ndim == 2
        assert NN.grid is g and NN.z == INTERFACES
        assert SS.grid is g and SS.z == INTERFACES
        sfx = _sfx(NN.all_values, SS.all_values, self.num.all_values, self.nuh.all_values)
        call("getm_keps_advance" + sfx, g.nx_, g.ny_, g.nz, g.halox, g.haloy, ctypes.addressof(self.params),
             float(timestep), g.mask.all_values.data_ptr(), g.hn.all_values.data_ptr(),
             ustar_s.all_values.data_ptr(), ustar_b.all_values.data_ptr(), z0s.all_values.data_ptr(),
             z0b.all_values.data_ptr(), NN.all_values.data_ptr(), SS.all_values.data_ptr(),
             self.tke.all_values.data_ptr(), self.eps.all_values.data_ptr(), self.L.all_values.data_ptr(),
             self.num.all_values.data_ptr(), self.nuh.all_values.data_ptr(), self._work.data_ptr(),
             torch.cuda.current_stream().cuda_stream)
        # viscosity at the open boundaries from the nearest interior point
        # (vertical_mixing.py:182-186): it is interpolated to the velocity
        # points just inside, and SS is not defined on the boundary
        if self._ob is not None:
            self._ob.update_zero_gradient(self.num)
