"""Device-resident grids and arrays (the counterparts of pygetm.core.Grid/Array).

A ``Grid`` holds one staggered grid of a domain on the GPU as torch tensors in
pygetm's layout ([k][j][i], halos included) plus a C-ABI grid handle through
which the CUDA kernels read its metrics.  An ``Array`` is a field on a grid:
a tensor with the grid it lives on and its vertical staggering
(python/pygetm/core.py:655-1163 for the reference semantics of fill, interp,
isel and the halo/mirror hooks).

One GPU holds one whole domain, so halo exchanges (update_halos*) are no-ops;
periodic domains are not supported.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from .domain import FILL_VALUE, HostGrid

CENTERS = 1  # python/pygetm/constants.py:6
INTERFACES = 2  # python/pygetm/constants.py:7


class Array:
    """A field on a ``Grid``; ``all_values`` is the full tensor with halos."""

    __slots__ = ("grid", "_all", "z", "fill_value", "name", "attrs")

    def __init__(self, grid: "Grid", all_values: torch.Tensor, z=False, fill_value=FILL_VALUE, name: Optional[str] = None):
        self.grid = grid
        self._all = all_values
        self.z = z
        self.fill_value = fill_value
        self.name = name
        self.attrs = {}

    @property
    def all_values(self) -> torch.Tensor:
        return self._all

    @all_values.setter
    def all_values(self, value):
        assert value is self._all

    @property
    def values(self) -> torch.Tensor:
        """Interior view (no halos)."""
        return self._all[self.grid.interior]

    @property
    def ndim(self) -> int:
        return self._all.ndim

    @property
    def shape(self):
        return tuple(self._all.shape)

    @property
    def dtype(self):
        return self._all.dtype

    def fill(self, value):
        """python/pygetm/core.py:901-911: set everywhere, then land to fill_value."""
        self._all[...] = value
        if self.fill_value is not None and self.ndim > 0:
            self._all[..., self.grid.land] = self.fill_value

    def isel(self, z: int) -> "Array":
        return Array(self.grid, self._all[z], z=False, fill_value=self.fill_value)

    def interp(self, target, z=None) -> "Array":
        """python/pygetm/core.py:940-972"""
        if not isinstance(target, Array):
            target = target.array(z=self.z if z is None else z, dtype=self.dtype)
        src = self._all
        tgt = target._all
        if self.grid is target.grid:
            if self.z == INTERFACES and target.z == CENTERS:
                interp_z(src, tgt, 0)
            elif self.z == CENTERS and target.z == INTERFACES:
                interp_z(src, tgt, 1)
        else:
            self.grid.interpolate(target.grid, src, tgt)
        return target

    # one subdomain per GPU: nothing to exchange
    def update_halos(self, *args, **kwargs):
        pass

    def update_halos_start(self, *args, **kwargs):
        pass

    def update_halos_finish(self, *args, **kwargs):
        pass

    def mirror(self, target: Optional["Array"] = None):
        """Open-boundary mirroring; closed domains have nothing to mirror."""
        return None

    def __repr__(self):
        return f"Array({self.name or '?'}, grid={self.grid.postfix}, shape={self.shape}, z={self.z})"


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _sfx_storage(velocities, fields):
    """Entry-point suffix from the velocity (or diffusivity) tensors and the
    field tensors: '' (all FP64), '_f32' (all float) or '_f64s' (float
    velocities, FP64-stored fields: the mixed form with FP64 tracers)."""
    v, f = _sfx(*velocities), _sfx(*fields)
    if v == f:
        return v
    if v == "_f32" and f == "":
        return "_f64s"
    raise TypeError(f"unsupported combination: velocities {velocities[0].dtype}, fields {fields[0].dtype}")


def _sfx(*tensors):
    """Entry-point suffix for the tensors' type: '' (FP64) or '_f32'."""
    dt = tensors[0].dtype
    for x in tensors[1:]:
        if x.dtype != dt:
            raise TypeError(f"mixed dtypes {[y.dtype for y in tensors]} in one call")
    if dt == torch.float64:
        return ""
    if dt == torch.float32:
        return "_f32"
    raise TypeError(f"unsupported dtype {dt}")


def interp_x(s, t, offset):
    s3 = s if s.ndim == 3 else s.unsqueeze(0)
    _lib.call("getm_grid_interp_x" + _sfx(s, t), s3.shape[2], s3.shape[1], s3.shape[0], s.data_ptr(), t.data_ptr(),
              offset, _stream())


def interp_y(s, t, offset):
    s3 = s if s.ndim == 3 else s.unsqueeze(0)
    _lib.call("getm_grid_interp_y" + _sfx(s, t), s3.shape[2], s3.shape[1], s3.shape[0], s.data_ptr(), t.data_ptr(),
              offset, _stream())


def interp_z(s, t, offset):
    _lib.call("getm_grid_interp_z" + _sfx(s, t), s.shape[2], s.shape[1], s.shape[0], t.shape[0], s.data_ptr(),
              t.data_ptr(), offset, _stream())


def interp_xy(s, t, ioffset, joffset):
    s3 = s if s.ndim == 3 else s.unsqueeze(0)
    t3 = t if t.ndim == 3 else t.unsqueeze(0)
    _lib.call("getm_grid_interp_xy" + _sfx(s, t), s3.shape[2], s3.shape[1], t3.shape[2], t3.shape[1], s3.shape[0],
              s.data_ptr(), t.data_ptr(), ioffset, joffset, _stream())


class Grid:
    """Device copy of one ``HostGrid`` with its time-varying fields."""

    def __init__(self, host: HostGrid, device="cuda"):
        self.host = host
        self.device = torch.device(device)
        self.nx, self.ny, self.nz = host.nx, host.ny, host.nz
        self.nz_ = host.nz
        self.halox, self.haloy = host.halox, host.haloy
        self.nx_, self.ny_ = host.nx_, host.ny_
        self.imin, self.imax, self.jmin, self.jmax = host.imin, host.imax, host.jmin, host.jmax
        self.ioffset, self.joffset = host.ioffset, host.joffset
        self.postfix = host.postfix
        self.ugrid = self.vgrid = self.xgrid = None
        f64 = dict(dtype=torch.float64, device=self.device)

        def dev(a, dtype=torch.float64):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dtype, device=self.device)

        self.mask = Array(self, dev(host.mask, torch.int32), fill_value=0, name="mask" + self.postfix)
        for name in ("x", "y", "dx", "dy", "idx", "idy", "area", "iarea", "cor", "H", "z0b_min"):
            setattr(self, name, Array(self, dev(host.arrays[name]), name=name + self.postfix))
        self.land = dev(host.land, torch.bool)
        self.water = ~self.land
        self.water_contact = dev(host.water_contact, torch.bool)
        shape2 = (self.ny_, self.nx_)
        self.D = Array(self, torch.full(shape2, FILL_VALUE, **f64), name="D" + self.postfix)
        self.D.all_values[self.water] = self.H.all_values[self.water]
        self.Dclip = self.D
        self.z0b = Array(self, self.z0b_min.all_values.clone(), name="z0b" + self.postfix)
        self.alpha = Array(self, torch.full(shape2, FILL_VALUE, **f64), name="alpha" + self.postfix)
        nzs = (self.nz,) + shape2
        self.hn = Array(self, torch.full(nzs, FILL_VALUE, **f64), z=CENTERS, name="hn" + self.postfix)
        Hu = dev(host.H_unmasked)
        self.zc = Array(self, (-Hu).expand(nzs).clone(), z=CENTERS, name="zc" + self.postfix)
        self.zf = Array(self, (-Hu).expand((self.nz + 1,) + shape2).clone(), z=INTERFACES, name="zf" + self.postfix)
        self.ho = None
        self.z = self.zo = self.zin = self.zio = None
        self._work = self.array(fill_value=float("nan"))
        # C-ABI grid handle (create_grid of python/src/wrapper.F90:48)
        h = ctypes.c_void_p()
        _lib.call("getm_create_grid", self.imin, self.imax, self.jmin, self.jmax, 1, max(self.nz, 1),
                  self.halox, self.haloy, ctypes.byref(h))
        self.handle = h
        for name in ("mask", "dx", "dy", "idx", "idy", "iarea", "area"):
            _lib.call("getm_grid_set_array", h, name.encode(), getattr(self, name).all_values.data_ptr())

    def float_metrics(self):
        """Make the float copies of the metrics (read by the mixed form's
        kernels) on the current stream, after the uploads above, waiting for
        that stream only."""
        _lib.call("getm_grid_float_metrics", self.handle, torch.cuda.current_stream(self.device).cuda_stream)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.release("getm_grid_finalize", h)
            except Exception:
                pass

    @property
    def interior(self):
        return (Ellipsis, slice(self.haloy, self.haloy + self.ny), slice(self.halox, self.halox + self.nx))

    def array(self, fill=None, z=False, fill_value=FILL_VALUE, dtype=torch.float64, name=None) -> Array:
        nlev = {False: None, None: None, CENTERS: self.nz, INTERFACES: self.nz + 1}[z]
        shape = (self.ny_, self.nx_) if nlev is None else (nlev, self.ny_, self.nx_)
        a = Array(self, torch.empty(shape, dtype=dtype, device=self.device), z=z, fill_value=fill_value, name=name)
        # Array.create (python/pygetm/core.py:853-900): an explicit fill is
        # written everywhere (land included); otherwise the fill value is.
        if fill is not None:
            a.all_values.fill_(fill)
        else:
            a.all_values.fill_(fill_value if fill_value is not None else 0)
        return a

    def interpolate(self, target: "Grid", src: torch.Tensor, tgt: torch.Tensor):
        """core.Grid.interpolator (python/pygetm/core.py:407-462)."""
        a, b = self, target
        if a.ioffset == b.ioffset + 1 and a.joffset == b.joffset:
            interp_x(src, tgt, 1)
        elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset:
            interp_x(src, tgt, 0)
        elif a.joffset == b.joffset + 1 and a.ioffset == b.ioffset:
            interp_y(src, tgt, 1)
        elif a.joffset == b.joffset - 1 and a.ioffset == b.ioffset:
            interp_y(src, tgt, 0)
        elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset - 1:
            interp_xy(src, tgt, 0, 0)
        elif a.ioffset == b.ioffset + 1 and a.joffset == b.joffset + 1:
            interp_xy(src, tgt, 1, 1)
        elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset + 1:
            interp_xy(src, tgt, 0, 1)
        elif a.ioffset == b.ioffset + 1 and a.joffset == b.joffset - 1:
            interp_xy(src, tgt, 1, 0)
        elif a.ioffset == b.ioffset - 2 and a.joffset == b.joffset:
            tgt[..., 0:-1].copy_(src[..., 1:])
        elif a.ioffset == b.ioffset and a.joffset == b.joffset - 2:
            tgt[..., 0:-1, :].copy_(src[..., 1:, :])
        else:
            raise NotImplementedError(f"Cannot interpolate from grid {a.postfix} to grid {b.postfix}")

    def all_grids(self):
        out = [self]
        for c in (self.ugrid, self.vgrid, self.xgrid):
            if c is not None:
                for g in c.all_grids():
                    if all(g is not o for o in out):
                        out.append(g)
        return out


def make_grids(T_host: HostGrid, device="cuda") -> Grid:
    """Device Grid tree mirroring a HostGrid tree (shared children stay shared)."""
    made = {}

    def mk(hg):
        if hg is None:
            return None
        if id(hg) in made:
            return made[id(hg)]
        g = Grid(hg, device)
        made[id(hg)] = g
        g.ugrid, g.vgrid, g.xgrid = mk(hg.ugrid), mk(hg.vgrid), mk(hg.xgrid)
        return g

    return mk(T_host)
