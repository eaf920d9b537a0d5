"""Drop-in GPU counterpart of ``pygetm.operators`` (python/pygetm/operators.py).

Same classes, constructor arguments, methods, attributes (``h``, ``D``,
``ufirst``, ``halo1``/``halo2``) and assertions.  The split sequences run as
fused launches of libgetm_gb300 (one kernel per directional stage for all
tracers of a batch) on the current torch CUDA stream; single directional
passes (``u_3d`` ...) remain available with the reference's in-place
semantics.
"""

from __future__ import annotations

import ctypes
import enum
from typing import Callable, Iterable, Optional

import torch

from . import _lib
from ._lib import call
from .core import CENTERS, INTERFACES, Array, Grid, _sfx, _sfx_storage  # noqa: F401


class AdvectionScheme(enum.IntEnum):
    """python/pygetm/operators.py:11-18"""

    HSIMT = 1
    MUSCL = 2
    P2_PDM = 3
    SPLMAX13 = 4
    SUPERBEE = 5
    UPSTREAM = 6
    DEFAULT = SUPERBEE


class AdvectionSplit(enum.Enum):
    """python/pygetm/operators.py:21-24"""

    FULL = 1
    HALF = 2
    HALF_ALWAYS = 3


class Neighbor(enum.IntEnum):
    """Halo-exchange directions (python/pygetm/parallel.py); no-ops on one GPU."""

    LEFT_AND_RIGHT = 1
    TOP_AND_BOTTOM = 2


def _s():
    return torch.cuda.current_stream().cuda_stream


def _p(a):
    if a is None:
        return None
    return (a.all_values if isinstance(a, Array) else a).data_ptr()


class Advection:
    """pygetm.operators.Advection (operators.py:27-193, pyx:198-261)."""

    def __init__(self, grid: Grid, scheme: AdvectionScheme = AdvectionScheme.DEFAULT,
                 split_2d: AdvectionSplit = AdvectionSplit.HALF, increments_2d: str = "float64"):
        """``increments_2d``: arithmetic of ``__call__`` (2D advection of a
        float64 field): "float64", the reference arithmetic, or "float32",
        the mixed form's increment form (float64 storage and updates)."""
        if increments_2d not in ("float64", "float32"):
            raise ValueError(f"increments_2d must be 'float64' or 'float32', not {increments_2d!r}")
        self._call_2d = "getm_advection_2d" if increments_2d == "float64" else "getm_advection_2d_mixed"
        self.grid = grid
        self.ugrid = grid.ugrid
        self.vgrid = grid.vgrid
        self.scheme = AdvectionScheme(scheme)
        h = ctypes.c_void_p()
        call("getm_advection_create", int(self.scheme), grid.handle, ctypes.byref(h))
        self.p = h
        # work array for layer heights during 3D advection; its first layer is
        # the column height D of 2D advection (pyx:216-219)
        self.h = torch.empty((max(grid.nz_, 1), grid.ny_, grid.nx_), dtype=torch.float64, device=grid.device)
        self.D = self.h[0, ...]
        self.ufirst = False
        self.split_2d = split_2d

    def __del__(self):
        p = getattr(self, "p", None)
        if p is not None and p.value:
            try:
                _lib.release("getm_advection_finalize", p)
            except Exception:
                pass

    @property
    def ufirst(self) -> bool:
        return self._ufirst

    @ufirst.setter
    def ufirst(self, value: bool):
        self._ufirst = value
        self.halo1 = Neighbor.LEFT_AND_RIGHT
        self.halo2 = Neighbor.TOP_AND_BOTTOM
        if not self._ufirst:
            self.halo1, self.halo2 = self.halo2, self.halo1

    # ---- single directional passes (pyx:234-261) ---------------------------
    def u_2d(self, u: Array, timestep: float, var: Array, Ah: Optional[Array] = None):
        call("getm_advection_uv_calculate", 1, 1, self.p, self.grid.handle, self.ugrid.handle, _p(u), _p(Ah),
             float(timestep), self.h.data_ptr(), _p(self.ugrid.D), _p(var), _s())

    def v_2d(self, v: Array, timestep: float, var: Array, Ah: Optional[Array] = None):
        call("getm_advection_uv_calculate", 2, 1, self.p, self.grid.handle, self.vgrid.handle, _p(v), _p(Ah),
             float(timestep), self.h.data_ptr(), _p(self.vgrid.D), _p(var), _s())

    def u_3d(self, u: Array, timestep: float, var: Array, Ah: Optional[Array] = None):
        call("getm_advection_uv_calculate", 1, var.all_values.shape[0], self.p, self.grid.handle, self.ugrid.handle,
             _p(u), _p(Ah), float(timestep), self.h.data_ptr(), _p(self.ugrid.hn), _p(var), _s())

    def v_3d(self, v: Array, timestep: float, var: Array, Ah: Optional[Array] = None):
        call("getm_advection_uv_calculate", 2, var.all_values.shape[0], self.p, self.grid.handle, self.vgrid.handle,
             _p(v), _p(Ah), float(timestep), self.h.data_ptr(), _p(self.vgrid.hn), _p(var), _s())

    def w_3d(self, w: Array, w_var: Array, timestep: float, var: Array):
        call("getm_advection_w_calculate", self.p, self.grid.handle, _p(w), _p(w_var), float(timestep),
             self.h.data_ptr(), _p(var), _s())

    # ---- split sequences -----------------------------------------------------
    def __call__(self, u: Array, v: Array, timestep: float, var: Array, Ah_u: Optional[Array] = None,
                 Ah_v: Optional[Array] = None, skip_initial_halo_exchange: bool = False):
        """operators.py:52-93"""
        assert u.grid is self.ugrid and not u.z
        assert v.grid is self.vgrid and not v.z
        assert var.grid is self.grid and not var.z
        assert Ah_u is None or (Ah_u.grid is self.ugrid and not Ah_u.z)
        assert Ah_v is None or (Ah_v.grid is self.vgrid and not Ah_v.z)
        self.D.copy_(self.grid.D.all_values)
        call(self._call_2d, self.p, self.grid.handle, self.ugrid.handle, self.vgrid.handle, int(self._ufirst),
             self.split_2d.value, _p(u), _p(v), _p(Ah_u), _p(Ah_v), float(timestep), self.D.data_ptr(),
             _p(self.ugrid.D), _p(self.vgrid.D), _p(var), _s())

    def apply_3d(self, u: Array, v: Array, w: Array, timestep: float, var: Array, Ah_u: Optional[Array] = None,
                 Ah_v: Optional[Array] = None, new_h: bool = False, skip_initial_halo_exchange: bool = False,
                 w_var: Optional[Array] = None):
        """operators.py:95-133"""
        if w_var is None:
            w_var = w
        assert u.grid is self.ugrid and u.z == CENTERS
        assert v.grid is self.vgrid and v.z == CENTERS
        assert w.grid is self.grid and w.z == INTERFACES
        assert w_var.grid is self.grid and w_var.z == INTERFACES
        assert var.grid is self.grid and var.z == CENTERS
        assert Ah_u is None or (Ah_u.grid is self.ugrid and not Ah_u.z)
        assert Ah_v is None or (Ah_v.grid is self.vgrid and not Ah_v.z)
        self._batch(u, v, w, timestep, [var], [w_var], Ah_u, Ah_v, new_h)

    def apply_3d_batch(self, u: Array, v: Array, w: Array, timestep: float, vars: Iterable[Array],
                       Ah_u: Optional[Array] = None, Ah_v: Optional[Array] = None, new_h: bool = False,
                       skip_initial_halo_exchange: bool = False,
                       get_w: Optional[Callable[[Array], Array]] = None):
        """operators.py:135-193"""
        vars = list(vars)
        assert u.grid is self.ugrid and u.z == CENTERS
        assert v.grid is self.vgrid and v.z == CENTERS
        assert w.grid is self.grid and w.z == INTERFACES
        for var in vars:
            assert var.grid is self.grid and var.z == CENTERS
        w_vars = []
        for var in vars:
            w_var = w if get_w is None else get_w(var)
            assert w_var.grid is self.grid and w_var.z == INTERFACES
            w_vars.append(w_var)
        self._batch(u, v, w, timestep, vars, w_vars, Ah_u, Ah_v, new_h)

    def _batch(self, u, v, w, timestep, vars, w_vars, Ah_u, Ah_v, new_h):
        self.h.copy_((self.grid.hn if new_h else self.grid.ho).all_values)
        wv = _lib.ptr_array([_p(x) for x in w_vars])
        vv = _lib.ptr_array([_p(x) for x in vars])
        sfx = _sfx_storage([u.all_values, v.all_values, w.all_values] + [x.all_values for x in w_vars],
                           [x.all_values for x in vars])
        call("getm_advection_apply_3d_batch" + sfx, self.p, self.grid.handle, self.ugrid.handle, self.vgrid.handle,
             int(self._ufirst), _p(u), _p(v), _p(w), wv, _p(Ah_u), _p(Ah_v), float(timestep), self.h.data_ptr(),
             _p(self.ugrid.hn), _p(self.vgrid.hn), len(vars), vv, _s())

    def status(self) -> int:
        """GETM_ERR_ITERS (3) if any column needed more than 200 sub-steps."""
        return _lib.lib.getm_advection_get_status(self.p, _s())


class VerticalAdvection:
    """pygetm.operators.VerticalAdvection (operators.py:196-215, pyx:263-286)."""

    def __init__(self, grid: Grid, scheme: AdvectionScheme = AdvectionScheme.DEFAULT):
        self.grid = grid
        h = ctypes.c_void_p()
        call("getm_advection_create", int(scheme), grid.handle, ctypes.byref(h))
        self.p = h
        self.h = torch.empty((grid.nz_, grid.ny_, grid.nx_), dtype=torch.float64, device=grid.device)

    def __del__(self):
        p = getattr(self, "p", None)
        if p is not None and p.value:
            try:
                _lib.release("getm_advection_finalize", p)
            except Exception:
                pass

    def w_3d(self, w: Array, w_var: Array, timestep: float, var: Array):
        call("getm_advection_w_calculate", self.p, self.grid.handle, _p(w), _p(w_var), float(timestep),
             self.h.data_ptr(), _p(var), _s())

    def __call__(self, w: Array, w_var: Array, timestep: float, var: Array, new_h: bool = False):
        assert w.grid is self.grid and w.z == INTERFACES
        assert w_var.grid is self.grid and w_var.z == INTERFACES
        self.h.copy_((self.grid.hn if new_h else self.grid.ho).all_values)
        self.w_3d(w, w_var, timestep, var)


class VerticalDiffusion:
    """pygetm.operators.VerticalDiffusion (operators.py:218-230, pyx:288-316)."""

    def __init__(self, grid: Grid, cnpar: float = 1.0):
        self.grid = grid
        self.cnpar = cnpar
        self._work = {}  # dtype -> workspace of the fused column solve
        h = ctypes.c_void_p()
        call("getm_vertical_diffusion_create", grid.handle, ctypes.byref(h))
        self.p = h

    def __del__(self):
        p = getattr(self, "p", None)
        if p is not None and p.value:
            try:
                _lib.release("getm_vertical_diffusion_finalize", p)
            except Exception:
                pass

    def prepare(self, nuh: Array, timestep: float, molecular: float = 0.0, use_ho: bool = False):
        g = nuh.grid
        ho = g.ho if use_ho else g.hn
        call("getm_vertical_diffusion_prepare", self.p, g.nx_, g.ny_, g.nz_, float(molecular), _p(nuh), float(timestep),
             float(self.cnpar), _p(g.mask), _p(ho), _p(g.hn), _s())

    def apply(self, var: Array, ea2: Optional[Array] = None, ea4: Optional[Array] = None, use_ho: bool = False):
        g = var.grid
        ho = g.ho if use_ho else g.hn
        call("getm_vertical_diffusion_apply", self.p, g.nx_, g.ny_, g.nz_, _p(g.mask), _p(ho), _p(g.hn), _p(var),
             _p(ea2), _p(ea4), _s())

    def __call__(self, nuh: Array, timestep: float, var: Array, molecular: float = 0.0, ea2: Optional[Array] = None,
                 ea4: Optional[Array] = None, use_ho: bool = False):
        """prepare + apply, fused into one column sweep."""
        self.batch(nuh, timestep, [var], [molecular], [ea2], [ea4], use_ho)

    def batch(self, nuh: Array, timestep: float, vars, molecular, ea2s=None, ea4s=None, use_ho: bool = False):
        """Fused prepare+apply for several fields sharing nuh and thicknesses,
        each with its own molecular diffusivity and optional sources."""
        g = nuh.grid
        ho = g.ho if use_ho else g.hn
        n = len(vars)
        mol = (ctypes.c_double * n)(*[float(m) for m in molecular])
        vv = _lib.ptr_array([_p(v) for v in vars])
        e2 = _lib.ptr_array([_p(e) for e in ea2s]) if ea2s is not None and any(e is not None for e in ea2s) else None
        e4 = _lib.ptr_array([_p(e) for e in ea4s]) if ea4s is not None and any(e is not None for e in ea4s) else None
        sfx = _sfx_storage([nuh.all_values], [v.all_values for v in vars])
        # elimination coefficients of the column solves (2 nz planes per field
        # solved at once, reused; the float solve takes its fields in pairs),
        # in the solve's type (that of nuh)
        dt = nuh.all_values.dtype
        need = 2 * (2 if n > 1 and dt == torch.float32 else 1) * g.nz_ * g.ny_ * g.nx_
        w = self._work.get(dt)
        if w is None or w.numel() < need:
            w = self._work[dt] = torch.empty(need, dtype=dt, device=nuh.all_values.device)
        call("getm_vertical_diffusion_batch" + sfx, g.nx_, g.ny_, g.nz_, _p(g.mask), _p(nuh), float(timestep),
             float(self.cnpar), _p(ho), _p(g.hn), n, mol, vv, e2, e4, w.data_ptr(), _s())
