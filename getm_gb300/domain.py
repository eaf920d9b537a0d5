"""Host-side domain and staggered-grid construction.

This is set-up code (numpy, runs once per domain), not the time-step path.  It
reproduces how pygetm derives the eight staggered grids of a domain, because
the masks and metrics it produces decide which points every operator touches:

* the domain is described on a "supergrid" of shape (2*ny+1, 2*nx+1) holding T
  points at odd/odd, U at odd/even, V at even/odd and X (corner) points at
  even/even positions (python/pygetm/domain.py:426-584, 586-661);
* T, U, V, X grids and the momentum-advection grids UU, UV, VU, VV are strided
  views of that supergrid with the offsets of python/pygetm/domain.py:699-725;
* U/V/X masks are closed where a neighbouring T point is land
  (infer_UVX_masks2, python/pygetm/domain.py:918-941;
  close_flux_interfaces, python/pygetm/core.py:380-390) and water-contact flags
  are derived as in python/pygetm/core.py:392-405;
* freezing computes inverse metrics and fills land with FILL_VALUE
  (python/pygetm/core.py:328-378).

Arrays use the C layout [j][i] with a halo of ``halox``/``haloy`` cells, the
layout pygetm hands to its Fortran kernels (python/_pygetm.pyx:104-114).
Only single-subdomain (one GPU) layouts are built: there is no MPI tiling.
"""

from __future__ import annotations

import enum
from typing import Dict, Optional

import numpy as np

FILL_VALUE = -2e20  # python/pygetm/constants.py:16
GRAVITY = 9.81  # python/pygetm/constants.py:4
RHO0 = 1025.0  # python/pygetm/constants.py:3


OMEGA = 2.0 * np.pi / 86164.0  # rotation rate of the earth (python/pygetm/domain.py:55-57)
DEG2RAD = np.pi / 180


def coriolis(lat):
    """Coriolis parameter for latitude (python/pygetm/domain.py:60-69)."""
    return (2.0 * OMEGA) * np.sin(DEG2RAD * np.asarray(lat, dtype=float))


class EdgeTreatment(enum.Enum):
    """How supergrid edges are filled (python/pygetm/domain.py:19-24)."""

    MISSING = enum.auto()
    CLAMP = enum.auto()
    PERIODIC = enum.auto()
    EXTRAPOLATE = enum.auto()


def _expand_2d(source, edges_x, edges_y, missing_value=np.nan, dtype=None):
    """Pad a 2D array by one cell on each side (python/pygetm/domain.py:97-142)."""
    source = np.asarray(source)
    out = np.empty(
        source.shape[:-2] + (source.shape[-2] + 2, source.shape[-1] + 2),
        dtype=dtype or source.dtype,
    )
    out[..., 1:-1, 1:-1] = source
    for axis, edges in ((-1, edges_x), (-2, edges_y)):
        first = [slice(None)] * out.ndim
        last = [slice(None)] * out.ndim

        def idx(k):
            s = [slice(None)] * out.ndim
            s[axis] = k
            return tuple(s)

        if edges == EdgeTreatment.EXTRAPOLATE:
            out[idx(0)] = 2 * out[idx(1)] - out[idx(2)]
            out[idx(-1)] = 2 * out[idx(-2)] - out[idx(-3)]
        elif edges == EdgeTreatment.CLAMP:
            out[idx(0)] = out[idx(1)]
            out[idx(-1)] = out[idx(-2)]
        elif edges == EdgeTreatment.PERIODIC:
            out[idx(0)] = out[idx(-2)]
            out[idx(-1)] = out[idx(1)]
        else:
            out[idx(0)] = missing_value
            out[idx(-1)] = missing_value
        del first, last
    return out


def _centers_to_supergrid_1d(source, edges, missing_value=np.nan):
    """python/pygetm/domain.py:66-95"""
    source = np.asarray(source, dtype=float)
    out = np.empty((source.size * 2 + 1,))
    out[1::2] = source
    out[2:-2:2] = 0.5 * (source[1:] + source[:-1])
    if edges == EdgeTreatment.PERIODIC:
        out[0] = out[-1] = 0.5 * (out[1] + out[-2])
    elif edges == EdgeTreatment.EXTRAPOLATE:
        out[0] = 2 * out[1] - out[2]
        out[-1] = 2 * out[-2] - out[-3]
    elif edges == EdgeTreatment.CLAMP:
        out[0] = out[1]
        out[-1] = out[-2]
    else:
        out[0] = out[-1] = missing_value
    return out


def _centers_to_supergrid_2d(source, edges_x, edges_y, missing_value=np.nan, dtype=None):
    """python/pygetm/domain.py:145-183.  For an integer dtype the averages are
    truncated on assignment, as numpy does in the reference."""
    source = np.asarray(source)
    ny, nx = source.shape
    ex = _expand_2d(source, edges_x, edges_y, missing_value, dtype)
    out = np.empty((ny * 2 + 1, nx * 2 + 1), dtype=ex.dtype)
    out[1::2, 1::2] = ex[1:-1, 1:-1]
    out[::2, ::2] = (ex[:-1, :-1] + ex[1:, :-1] + ex[:-1, 1:] + ex[1:, 1:]) / 4.0
    out[::2, 1::2] = (ex[:-1, 1:-1] + ex[1:, 1:-1]) / 2.0
    out[1::2, ::2] = (ex[1:-1, :-1] + ex[1:-1, 1:]) / 2.0
    return out


def _interfaces_to_supergrid_1d(source):
    """python/pygetm/domain.py:186-199"""
    source = np.asarray(source, dtype=float)
    out = np.empty((source.size * 2 - 1,))
    out[0::2] = source
    out[1::2] = 0.5 * (source[1:] + source[:-1])
    return out


class HostGrid:
    """One staggered grid of a domain, as numpy arrays with halos.

    Mirrors the static part of ``pygetm.core.Grid`` (python/pygetm/core.py:106):
    index extent, offsets on the supergrid, masks and metrics.  Time-varying
    fields (D, hn, zc, ...) live on the device-side grid.
    """

    STATIC = ("x", "y", "dx", "dy", "area", "cor", "H", "mask", "z0b_min")

    def __init__(self, nx, ny, nz, halox, haloy, postfix, ioffset, joffset, overlap=0):
        self.nx, self.ny, self.nz = nx + overlap, ny + overlap, nz
        self.halox, self.haloy = halox, haloy
        self.nx_, self.ny_ = self.nx + 2 * halox, self.ny + 2 * haloy
        self.postfix = postfix
        self.ioffset, self.joffset, self.overlap = ioffset, joffset, overlap
        self.ugrid: Optional[HostGrid] = None
        self.vgrid: Optional[HostGrid] = None
        self.xgrid: Optional[HostGrid] = None
        self.arrays: Dict[str, np.ndarray] = {}

    # Fortran 1-based interior bounds as create_grid receives them
    # (python/_pygetm.pyx:166-172).  X is created with istart=jstart=0.
    @property
    def imin(self):
        return 0 if self.postfix == "x" else 1

    @property
    def jmin(self):
        return self.imin

    @property
    def imax(self):
        return self.imin + self.nx - 1

    @property
    def jmax(self):
        return self.jmin + self.ny - 1

    @property
    def interior(self):
        return (Ellipsis, slice(self.haloy, self.haloy + self.ny), slice(self.halox, self.halox + self.nx))

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def empty(self, fill=FILL_VALUE, dtype=float, nz=None):
        shape = (self.ny_, self.nx_) if nz is None else (nz, self.ny_, self.nx_)
        return np.full(shape, fill, dtype=dtype)

    def children(self):
        return [g for g in (self.ugrid, self.vgrid, self.xgrid) if g is not None]

    def all_grids(self):
        out = [self]
        for c in self.children():
            for g in c.all_grids():
                if all(g is not o for o in out):
                    out.append(g)
        return out

    def close_flux_interfaces(self):
        """python/pygetm/core.py:380-390"""
        tmask = self.mask
        umask = (tmask[:, :-1] == 0) | (tmask[:, 1:] == 0)
        vmask = (tmask[:-1, :] == 0) | (tmask[1:, :] == 0)
        umask &= self.ugrid.mask[:, :-1] == 1
        vmask &= self.vgrid.mask[:-1, :] == 1
        self.ugrid.mask[:, :-1][umask] = 0
        self.vgrid.mask[:-1, :][vmask] = 0

    def infer_water_contact(self):
        """python/pygetm/core.py:392-405"""
        tmask = self.mask
        for child, wc in (
            (self.ugrid, (tmask[:, :-1] != 0) | (tmask[:, 1:] != 0)),
            (self.vgrid, (tmask[:-1, :] != 0) | (tmask[1:, :] != 0)),
        ):
            contact = np.zeros_like(child.mask, dtype=bool)
            if child is self.ugrid:
                contact[:, :-1] = wc
            else:
                contact[:-1, :] = wc
            child.water_contact = contact

    def freeze(self):
        """python/pygetm/core.py:328-378 (derived metrics, land fill)."""
        with np.errstate(divide="ignore"):
            self.arrays["iarea"] = 1.0 / self.area
            self.arrays["idx"] = 1.0 / self.dx
            self.arrays["idy"] = 1.0 / self.dy
        self.land = self.mask == 0
        self.water = ~self.land
        if not hasattr(self, "water_contact"):
            self.water_contact = self.water
        # Vertical coordinates start out at the (unmasked) bottom.
        self.H_unmasked = self.H.copy()
        self.H[self.land] = FILL_VALUE
        self.z0b_min[self.land] = FILL_VALUE


class Domain:
    """Rectangular domain on a supergrid (python/pygetm/domain.py:426-584).

    Args mirror ``pygetm.domain.Domain``: x/y at cell centres (1D or 2D), mask
    (0 land, 1 water), bathymetric depth H, bottom roughness z0 and Coriolis
    parameter f, each given at centres (ny, nx) or as a scalar.
    """

    def __init__(self, nx, ny, *, x, y, mask=1, H=None, z0=0.0, f=None, lat=None, periodic_x=False,
                 periodic_y=False):
        if f is None and lat is None:
            raise Exception("Either lat of f must be provided to determine the Coriolis parameter.")
        if f is None:
            f = coriolis(lat)
        if periodic_x or periodic_y:
            raise NotImplementedError("periodic domains are not supported")
        self.nx, self.ny = nx, ny
        self.periodic_x, self.periodic_y = periodic_x, periodic_y
        self._x = self._map(x, EdgeTreatment.EXTRAPOLATE)
        self._y = self._map(y, EdgeTreatment.EXTRAPOLATE)
        self._f = self._map(f)
        self._mask = self._map(mask, missing_value=0, dtype=int)
        self._H = self._map(H, EdgeTreatment.CLAMP)
        self._z0 = self._map(z0)
        x_ex = _expand_2d(self._x, EdgeTreatment.EXTRAPOLATE, EdgeTreatment.EXTRAPOLATE)
        y_ex = _expand_2d(self._y, EdgeTreatment.EXTRAPOLATE, EdgeTreatment.EXTRAPOLATE)
        dx_x = x_ex[1:-1, 2:] - x_ex[1:-1, :-2]
        dy_x = y_ex[1:-1, 2:] - y_ex[1:-1, :-2]
        dx_y = x_ex[2:, 1:-1] - x_ex[:-2, 1:-1]
        dy_y = y_ex[2:, 1:-1] - y_ex[:-2, 1:-1]
        self._dx = np.hypot(dx_x, dy_x)
        self._dy = np.hypot(dx_y, dy_y)
        self._area = self._dx * self._dy
        from .open_boundaries import OpenBoundaries

        self.open_boundaries = OpenBoundaries(nx, ny)

    @property
    def mask(self):
        """Mask at T points (a writable view into the supergrid)."""
        return self._mask[1::2, 1::2]

    @mask.setter
    def mask(self, value):
        self._mask[...] = self._map(value, missing_value=0, dtype=int)

    @property
    def H(self):
        return self._H[1::2, 1::2]

    def _map(self, values, edges=EdgeTreatment.MISSING, missing_value=np.nan, dtype=float):
        """python/pygetm/domain.py:586-661"""
        target_shape = (self.ny * 2 + 1, self.nx * 2 + 1)
        if values is None:
            return None
        values = np.asarray(values)
        shape = (1,) * (2 - values.ndim) + values.shape
        if shape == (1, 1):
            mapped = np.array(values, dtype=dtype)
        elif shape[-1] in (1, self.nx) and shape[-2] in (1, self.ny):
            if shape[0] == 1:
                mapped = _centers_to_supergrid_1d(np.ravel(values), edges, missing_value)[np.newaxis, :]
            elif shape[1] == 1:
                mapped = _centers_to_supergrid_1d(np.ravel(values), edges, missing_value)[:, np.newaxis]
            else:
                mapped = _centers_to_supergrid_2d(values, edges, edges, missing_value, dtype)
        elif shape[-1] in (1, self.nx + 1) and shape[-2] in (1, self.ny + 1):
            if shape[0] == 1:
                mapped = _interfaces_to_supergrid_1d(np.ravel(values))[np.newaxis, :]
            else:
                mapped = _interfaces_to_supergrid_1d(np.ravel(values))[:, np.newaxis]
        else:
            mapped = np.asarray(values, dtype=dtype)
        return np.array(np.broadcast_to(mapped, target_shape), dtype=dtype)

    def infer_UVX_masks2(self):
        """python/pygetm/domain.py:918-941"""
        tmask = self._mask[1::2, 1::2]
        umask = self._mask[1::2, ::2]
        vmask = self._mask[::2, 1::2]
        xmask = self._mask[::2, ::2]
        ex = _expand_2d(tmask, EdgeTreatment.MISSING, EdgeTreatment.MISSING, missing_value=0)
        bad = (ex[1:-1, 1:] == 0) | (ex[1:-1, :-1] == 0)
        umask[bad & (umask == 1)] = 0
        bad = (ex[1:, 1:-1] == 0) | (ex[:-1, 1:-1] == 0)
        vmask[bad & (vmask == 1)] = 0
        bad = (ex[1:, 1:] == 0) | (ex[:-1, 1:] == 0) | (ex[1:, :-1] == 0) | (ex[:-1, :-1] == 0)
        xmask[bad] = 0

    def _populate(self, grid: HostGrid):
        """python/pygetm/domain.py:763-850 for a single subdomain."""
        ioff, joff = grid.ioffset % 2, grid.joffset % 2
        istart = (ioff - grid.ioffset) // 2
        jstart = (joff - grid.joffset) // 2
        nx_glob, ny_glob = self.nx + grid.overlap, self.ny + grid.overlap
        sources = dict(
            x=self._x, y=self._y, cor=self._f, dx=self._dx, dy=self._dy,
            area=self._area, mask=self._mask, H=self._H, z0b_min=self._z0,
        )
        for name, source in sources.items():
            dtype = int if name == "mask" else float
            fill = 0 if name == "mask" else FILL_VALUE
            target = grid.empty(fill, dtype)
            if grid.joffset > 1 or grid.ioffset > 1:
                source = _expand_2d(source, EdgeTreatment.MISSING, EdgeTreatment.MISSING, missing_value=fill, dtype=source.dtype)[1:, 1:]
            gv = source[joff::2, ioff::2]
            # global index g <-> subdomain index g + istart; local = sub + halo
            i0, j0 = istart + grid.halox, jstart + grid.haloy
            gi0, gj0 = max(0, -i0), max(0, -j0)
            ni = min(gv.shape[1] - gi0, grid.nx_ - (i0 + gi0))
            nj = min(gv.shape[0] - gj0, grid.ny_ - (j0 + gj0))
            target[j0 + gj0 : j0 + gj0 + nj, i0 + gi0 : i0 + gi0 + ni] = gv[gj0 : gj0 + nj, gi0 : gi0 + ni]
            grid.arrays[name] = target
        del nx_glob, ny_glob

    def create_grids(self, nz: int, halox: int = 2, haloy: int = 2, velocity_grids: int = 2) -> HostGrid:
        """python/pygetm/domain.py:663-761"""
        if self._H is None:
            raise Exception("Water depth at rest (H) has not been provided")
        self.infer_UVX_masks2()
        self.open_boundaries.adjust_mask(self._mask)

        def make(postfix, ioffset, joffset, overlap=0):
            g = HostGrid(self.nx, self.ny, nz, halox, haloy, postfix, ioffset, joffset, overlap)
            self._populate(g)
            return g

        U = V = X = UU = UV = VU = VV = None
        if velocity_grids > 1:
            UU = make("_uu_adv", 3, 1)
            UV = make("_uv_adv", 2, 2)
            VU = make("_vu_adv", 2, 2)
            VV = make("_vv_adv", 1, 3)
        if velocity_grids > 0:
            U = make("u", 2, 1)
            U.ugrid, U.vgrid = UU, UV
            V = make("v", 1, 2)
            V.ugrid, V.vgrid = VU, VV
            X = make("x", 0, 0, overlap=1)
        T = make("t", 1, 1)
        T.ugrid, T.vgrid, T.xgrid = U, V, X
        if velocity_grids > 0:
            T.infer_water_contact()
            T.close_flux_interfaces()
        if velocity_grids > 1:
            U.close_flux_interfaces()
            V.close_flux_interfaces()
            # no transport between velocity points just outside an open
            # boundary (python/pygetm/domain.py:752-762)
            UV.mask[:-1, :][(U.mask[:-1, :] == 4) & (U.mask[1:, :] == 4)] = 0
            VU.mask[:, :-1][(V.mask[:, :-1] == 4) & (V.mask[:, 1:] == 4)] = 0
        for g in T.all_grids():
            g.freeze()
        self.open_boundaries.initialize(T)
        return T

    def cfl_check(self) -> float:
        """Maximum stable 2D time step (python/pygetm/domain.py:852-884)."""
        dx = self._dx[1::2, 1::2]
        dy = self._dy[1::2, 1::2]
        D = self._H[1::2, 1::2]
        mask = (self._mask[1::2, 1::2] > 0) & (D > 0.0)
        denom2 = (2.0 * GRAVITY) * D * (dx**2 + dy**2)
        maxdts = dx * dy / np.sqrt(denom2, where=mask, out=np.ones_like(D))
        maxdts[~mask] = np.inf
        return float(maxdts.min())


def create_cartesian(x, y, *, interfaces: bool = False, **kwargs) -> Domain:
    """python/pygetm/domain.py:241-277 (without lon/lat)."""
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    if y.ndim == 1:
        y = y[:, np.newaxis]
    if interfaces:
        nx, ny = x.shape[-1] - 1, y.shape[0] - 1
    else:
        nx, ny = x.shape[-1], y.shape[0]
    return Domain(nx, ny, x=x, y=y, **kwargs)


def calculate_sigma(nz: int, ddl: float = 0.0, ddu: float = 0.0) -> np.ndarray:
    """Sigma layer fractions with optional zooming
    (python/pygetm/vertical_coordinates.py:70-90)."""
    if ddl <= 0.0 and ddu <= 0.0:
        return np.broadcast_to(1.0 / nz, (nz,)).copy()
    ddl, ddu = max(ddl, 0.0), max(ddu, 0.0)
    ga = np.linspace(0.0, 1.0, nz + 1)
    ga[1:-1] = np.tanh((ddl + ddu) * ga[1:-1] - ddl) + np.tanh(ddl)
    ga[1:-1] /= np.tanh(ddl) + np.tanh(ddu)
    dga = np.diff(ga)
    assert (dga > 0.0).all()
    return dga
