"""Open boundaries: description, masks and the per-point tables the kernels use.

Host-side counterpart of python/pygetm/open_boundaries.py for a single
subdomain.  A boundary is a row or column of T points (``add_by_index`` and
the ``add_*_boundary`` helpers, open_boundaries.py:562-660, with the same
validation); ``adjust_mask`` marks the supergrid as the reference does
(open_boundaries.py:665-707: T points on a boundary get mask 2, velocity
points between two boundary T points 3, velocity points just outside a
boundary 4).  ``initialize`` turns the collection into flat per-point tables
(halo-inclusive T indices, the inward direction, the condition of each point)
and the mirror index lists of open_boundaries.py:848-917, which the device
kernels in ``csrc/open_boundaries.cu`` consume.

Conditions (constants of python/pygetm/constants.py:9-14): ZERO_GRADIENT,
CLAMPED, FLATHER_ELEV, FLATHER_TRANSPORT for elevation (2D) and
ZERO_GRADIENT, CLAMPED, SPONGE for tracers (3D).  Prescribed elevations are
harmonic constituents (amplitude and phase per point, one frequency per
constituent) evaluated on the device from the model time, so a run with
tidal forcing stays graph-capturable.
"""

from __future__ import annotations

import enum
from typing import List, Optional

import numpy as np

ZERO_GRADIENT = 1
CLAMPED = 3
FLATHER_ELEV = 4
FLATHER_TRANSPORT = -4
SPONGE = 5

_VALID_2D = (ZERO_GRADIENT, CLAMPED, FLATHER_ELEV, FLATHER_TRANSPORT)
_VALID_3D = (ZERO_GRADIENT, CLAMPED, SPONGE)


class Side(enum.IntEnum):
    """python/pygetm/open_boundaries.py:37-41"""

    WEST = 1
    NORTH = 2
    EAST = 3
    SOUTH = 4


class OpenBoundary:
    """One boundary (python/pygetm/open_boundaries.py:44-107)."""

    def __init__(self, name: str, side: Side, l: int, mstart: int, mstop: int, type_2d: int, type_3d: int):
        self.name = name
        self.side = Side(side)
        self.l_glob = l
        self.mstart_glob = mstart
        self.mstop_glob = mstop
        self.mstep = 1 if mstop > mstart else -1
        self.type_2d = type_2d
        self.type_3d = type_3d
        self.inflow_sign = 1.0 if self.side in (Side.WEST, Side.SOUTH) else -1.0

    def __repr__(self) -> str:
        return f"OpenBoundary({self.name!r}, {self.side.name}, {self.l_glob}, {self.mstart_glob}, {self.mstop_glob})"

    def to_local_grid(self, halox: int, haloy: int):
        """Indices in the T grid including halos (one subdomain)."""
        ms = np.arange(self.mstart_glob, self.mstop_glob, self.mstep)
        self.np = ms.size
        if self.side in (Side.WEST, Side.EAST):
            self.i = np.full_like(ms, self.l_glob + halox)
            self.j = ms + haloy
        else:
            self.i = ms + halox
            self.j = np.full_like(ms, self.l_glob + haloy)


class OpenBoundaries:
    """The open boundaries of a domain (python/pygetm/open_boundaries.py:500-960)."""

    def __init__(self, nx: int, ny: int):
        self.nx, self.ny = nx, ny
        self._boundaries: List[OpenBoundary] = []
        self._frozen = False
        self.np = 0
        self.sponge_n = 3
        # harmonic constituents of the prescribed elevation: list of
        # (omega [rad/s], amplitude [np], phase [np]) set with set_tide
        self.constituents = []

    # ---- collection (open_boundaries.py:562-663) --------------------------
    def add_by_index(self, side: Side, l: int, mstart: int, mstop: int, type_2d: int, type_3d: int,
                     name: Optional[str] = None):
        """l, mstart, mstop are 0-based indices of T points of the global
        domain; mstop is the first index excluded."""
        assert not self._frozen, "The open boundary collection has already been initialized"
        if type_2d not in _VALID_2D:
            raise Exception(f"Unknown boundary type {type_2d} specified")
        if type_3d not in _VALID_3D:
            raise Exception(f"Unknown boundary type {type_3d} specified")
        side = Side(side)
        along_y = side in (Side.WEST, Side.EAST)
        l_max, m_max = (self.nx, self.ny) if along_y else (self.ny, self.nx)
        mstep = 1 if mstop > mstart else -1
        assert mstart >= 0 and mstart < m_max
        assert mstop - mstep > 0 and mstop - mstep < m_max
        assert mstart != mstop
        assert l >= 0 and l < l_max
        if name is None:
            name = str(len(self._boundaries))
        mmin = min(mstart, mstop - mstep)
        mmax = max(mstart, mstop - mstep)
        for b in self._boundaries:
            b_along_y = b.side in (Side.WEST, Side.EAST)
            bmin = min(b.mstart_glob, b.mstop_glob - b.mstep)
            bmax = max(b.mstart_glob, b.mstop_glob - b.mstep)
            if along_y == b_along_y:
                if l == b.l_glob:
                    overlap = min(mmax, bmax) + 1 - max(mmin, bmin)
                    if overlap > 0:
                        raise Exception(f"New boundary {name} overlaps in {overlap} points with existing boundary {b.name}")
            elif bmin <= l <= bmax and mmin <= b.l_glob <= mmax:
                i, j = (l, b.l_glob) if along_y else (b.l_glob, l)
                raise Exception(f"New boundary {name} crosses existing boundary {b.name} at i={i}, j={j}")
        self._boundaries.append(OpenBoundary(name, side, l, mstart, mstop, type_2d, type_3d))

    def add_top_boundary(self, name, j, istart, istop, type_2d, type_3d):
        self.add_by_index(Side.NORTH, j, istart, istop, type_2d, type_3d, name=name)

    def add_bottom_boundary(self, name, j, istart, istop, type_2d, type_3d):
        self.add_by_index(Side.SOUTH, j, istart, istop, type_2d, type_3d, name=name)

    def add_left_boundary(self, name, i, jstart, jstop, type_2d, type_3d):
        self.add_by_index(Side.WEST, i, jstart, jstop, type_2d, type_3d, name=name)

    def add_right_boundary(self, name, i, jstart, jstop, type_2d, type_3d):
        self.add_by_index(Side.EAST, i, jstart, jstop, type_2d, type_3d, name=name)

    def clear(self):
        self._boundaries.clear()

    def __len__(self):
        return len(self._boundaries)

    def __iter__(self):
        return iter(self._boundaries)

    def __getitem__(self, key):
        return self._boundaries[key]

    # ---- masks (open_boundaries.py:665-707) --------------------------------
    def adjust_mask(self, mask: np.ndarray):
        """Mark boundary T points 2, velocity points between boundary T points
        3 and velocity points just outside a boundary 4 on the supergrid mask
        of shape (1 + 2 ny, 1 + 2 nx)."""
        assert mask.shape == (1 + 2 * self.ny, 1 + 2 * self.nx)
        umask = mask[1::2, 0::2]
        vmask = mask[0::2, 1::2]
        tmask = mask[1::2, 1::2]
        for b in self._boundaries:
            l = b.l_glob
            mslice = slice(b.mstart_glob, b.mstop_glob, b.mstep)
            bdy_mask = tmask[mslice, l] if b.side in (Side.WEST, Side.EAST) else tmask[l, mslice]
            on_land = bdy_mask == 0
            if on_land.any():
                raise Exception(f"Open boundary {b.name}: {int(on_land.sum())} of {bdy_mask.size} points of this"
                                f" {b.side.name.capitalize()}ern boundary are on land")
            bdy_mask[:] = 2
            if b.side in (Side.WEST, Side.EAST):
                umask[mslice, l if b.side == Side.WEST else l + 1] = 4
            else:
                vmask[l if b.side == Side.SOUTH else l + 1, mslice] = 4
        umask[:, 1:-1][(tmask[:, :-1] == 2) & (tmask[:, 1:] == 2)] = 3
        vmask[1:-1, :][(tmask[:-1, :] == 2) & (tmask[1:, :] == 2)] = 3

    # ---- per-point tables (open_boundaries.py:709-917) ---------------------
    def initialize(self, T):
        """Freeze the collection and build the tables for HostGrid ``T``."""
        assert not self._frozen, "The open boundary collection has already been initialized"
        halox, haloy = T.halox, T.haloy
        ii, jj, t2, t3, sign, di, dj, side = [], [], [], [], [], [], [], []
        start = 0
        for b in self._boundaries:
            b.to_local_grid(halox, haloy)
            b.start, b.stop = start, start + b.np
            start += b.np
            ii.append(b.i)
            jj.append(b.j)
            t2.append(np.full(b.np, b.type_2d, dtype=np.int32))
            t3.append(np.full(b.np, b.type_3d, dtype=np.int32))
            sign.append(np.full(b.np, b.inflow_sign))
            inward = {Side.WEST: (1, 0), Side.EAST: (-1, 0), Side.SOUTH: (0, 1), Side.NORTH: (0, -1)}[b.side]
            di.append(np.full(b.np, inward[0], dtype=np.int32))
            dj.append(np.full(b.np, inward[1], dtype=np.int32))
            side.append(np.full(b.np, int(b.side), dtype=np.int32))
        cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)  # noqa: E731
        self.np = start
        self.i = cat(ii, np.int32)
        self.j = cat(jj, np.int32)
        self.type_2d = cat(t2, np.int32)
        self.type_3d = cat(t3, np.int32)
        self.inflow_sign = cat(sign, float)
        self.di = cat(di, np.int32)
        self.dj = cat(dj, np.int32)
        self.side = cat(side, np.int32)
        if self.np:
            assert (T.mask[self.j, self.i] == 2).all()
        self._configure_mirroring(T)
        self._frozen = True
        T.open_boundaries = self

    def _configure_mirroring(self, T):
        """Source and target points of the mirroring across boundaries on U
        and V grids and from T to U/V (open_boundaries.py:848-917).  Each list
        holds flat [j][i] indices into the halo-inclusive 2D planes."""
        nx_ = T.nx_
        U, V = T.ugrid, T.vgrid
        mU, mV, mTU, mTV = [], [], [], []
        for b in self._boundaries:
            if U is None:
                continue
            if b.side in (Side.WEST, Side.EAST):
                j_velout = np.arange(max(b.j.min() - 1, 0), b.j.max() + 1)
                i_velout = np.full_like(j_velout, b.i[0])
                mirror_mask = V.mask[j_velout, i_velout]
            else:
                i_velout = np.arange(max(b.i.min() - 1, 0), b.i.max() + 1)
                j_velout = np.full_like(i_velout, b.j[0])
                mirror_mask = U.mask[j_velout, i_velout]
            sel = mirror_mask == 3
            i_velout, j_velout = i_velout[sel], j_velout[sel]
            i_velin = i_velout + {Side.EAST: -1, Side.WEST: 1}.get(b.side, 0)
            j_velin = j_velout + {Side.NORTH: -1, Side.SOUTH: 1}.get(b.side, 0)
            i_in = b.i + {Side.EAST: -1}.get(b.side, 0)
            j_in = b.j + {Side.NORTH: -1}.get(b.side, 0)
            i_out = b.i + {Side.WEST: -1}.get(b.side, 0)
            j_out = b.j + {Side.SOUTH: -1}.get(b.side, 0)
            sel = (i_in >= 0) & (j_in >= 0) & (i_out >= 0) & (j_out >= 0)
            i_in, i_out, j_in, j_out = (a[sel] for a in (i_in, i_out, j_in, j_out))
            if b.side in (Side.WEST, Side.EAST):
                assert (U.mask[j_out, i_out] == 4).all()
                mU.append((i_in, j_in, i_out, j_out))
                mV.append((i_velin, j_velin, i_velout, j_velout))
                mTU.append((b.i, b.j, i_out, j_out))
            else:
                assert (V.mask[j_out, i_out] == 4).all()
                mV.append((i_in, j_in, i_out, j_out))
                mU.append((i_velin, j_velin, i_velout, j_velout))
                mTV.append((b.i, b.j, i_out, j_out))

        def pack(lst):
            if not lst:
                return np.zeros(0, np.int32), np.zeros(0, np.int32)
            src = np.concatenate([l_[1] * nx_ + l_[0] for l_ in lst]).astype(np.int32)
            tgt = np.concatenate([l_[3] * nx_ + l_[2] for l_ in lst]).astype(np.int32)
            return src, tgt

        self.mirror_U = pack(mU)
        self.mirror_V = pack(mV)
        self.mirror_TU = pack(mTU)
        self.mirror_TV = pack(mTV)

    # ---- prescribed elevation ---------------------------------------------
    def set_tide(self, omega: float, amplitude, phase=0.0):
        """Add a harmonic constituent of the prescribed boundary elevation:
        z_bdy += amplitude * cos(omega * t + phase), per boundary point."""
        amp = np.broadcast_to(np.asarray(amplitude, dtype=float), (self.np,)).copy()
        ph = np.broadcast_to(np.asarray(phase, dtype=float), (self.np,)).copy()
        self.constituents.append((float(omega), amp, ph))


class DeviceBoundaries:
    """Device copies of the point tables and the boundary operations of one
    simulation (one launch per boundary where the reference updates the
    boundaries in turn)."""

    def __init__(self, ob: OpenBoundaries, T, dtype3d):
        import torch

        dev = T.device
        self.T = T
        self.dtype3d = dtype3d

        def it(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)

        self.np = ob.np
        self.i, self.j = it(ob.i), it(ob.j)
        self.type_2d, self.type_3d = it(ob.type_2d), it(ob.type_3d)
        self.type_zero_gradient = it(np.full(ob.np, ZERO_GRADIENT))
        self.di, self.dj, self.side = it(ob.di), it(ob.dj), it(ob.side)
        self.sign = torch.from_numpy(ob.inflow_sign.astype(float)).to(dev)
        self.ranges = [(b.start, b.stop) for b in ob]
        self.nsponge = ob.sponge_n
        # prescribed elevation, and velocity (FLATHER_ELEV) or transport
        # (FLATHER_TRANSPORT) normal to the boundary, per point
        self.z = torch.zeros(self.np, dtype=torch.float64, device=dev)
        self.flow = torch.zeros(self.np, dtype=torch.float64, device=dev)
        self.constituents = [(om, torch.from_numpy(a).to(dev), torch.from_numpy(p).to(dev))
                             for om, a, p in ob.constituents]
        self.mirrors = {}
        nmax = 1
        for name in ("U", "V", "TU", "TV"):
            src, tgt = getattr(ob, "mirror_" + name)
            if np.unique(tgt).size != tgt.size:
                raise NotImplementedError("a mirror target appears twice")
            self.mirrors[name] = (it(src), it(tgt), int(src.size))
            nmax = max(nmax, int(src.size))
        # gather buffer of the two-phase mirror (nz levels of the 3D transports)
        self._mirror_work = torch.empty(nmax * max(T.nz, 1), dtype=torch.float64, device=dev)
        self.tracer_values = {}

    # ---- prescribed values --------------------------------------------------
    def prescribe(self, time):
        """z at the boundary from the harmonic constituents at model time
        ``time`` (0-d device tensor)."""
        if not self.constituents:
            return
        self.z.zero_()
        for om, amp, ph in self.constituents:
            self.z.add_(amp * (time * om + ph).cos())

    def init_tracer_values(self, tracers):
        """Prescribed tracer values (nz x np) default to the tracer's values
        at the boundary points when the run starts."""
        for tr in tracers:
            v = tr.all_values[:, self.j.long(), self.i.long()].contiguous()
            self.tracer_values[tr.name] = v

    # ---- operations ---------------------------------------------------------
    def update_elevation(self, sim):
        from . import _lib
        from ._pygetm import _p, _s

        T = self.T
        for s, e in self.ranges:
            _lib.call("getm_open_boundary_elevation", s, e, T.nx_, self.i.data_ptr(), self.j.data_ptr(),
                      self.type_2d.data_ptr(), self.di.data_ptr(), self.dj.data_ptr(), self.side.data_ptr(),
                      self.sign.data_ptr(), _p(T.H), _p(T.Dclip), _p(sim.momentum.U), _p(sim.momentum.V),
                      self.z.data_ptr(), self.flow.data_ptr(), float(sim.Dmin), _p(T.z), _s())

    def mirror(self, name, field):
        """core.Array.mirror with the pairs of grid ``name`` (U, V, TU, TV)."""
        from . import _lib
        from ._pygetm import _s
        import torch

        src, tgt, n = self.mirrors[name]
        if n == 0:
            return
        t = field.all_values if hasattr(field, "all_values") else field
        nlev = t.shape[0] if t.dim() == 3 else 1
        fn = "getm_mirror_f32" if t.dtype == torch.float32 else "getm_mirror"
        _lib.call(fn, n, src.data_ptr(), tgt.data_ptr(), nlev, t.shape[-1] * t.shape[-2], t.data_ptr(),
                  self._mirror_work.data_ptr(), _s())

    def update_depth(self, sim, z, zo):
        """Depths at the points just outside the boundaries (after the 2D
        depth update)."""
        from . import _lib
        from ._pygetm import _p, _s

        for name, g in (("TU", sim.U), ("TV", sim.V)):
            src, tgt, n = self.mirrors[name]
            if n:
                _lib.call("getm_open_boundary_depth", n, src.data_ptr(), tgt.data_ptr(), _p(z), _p(zo), _p(g.H),
                          _p(g.mask), float(sim.Dmin), float(sim.Dcrit), _p(g._work), _p(g.D), _p(g.alpha), _s())

    def update_zero_gradient(self, field):
        """ArrayOpenBoundaries.update of an array whose boundaries are all
        ZERO_GRADIENT (the turbulent viscosity, python/pygetm/vertical_mixing.py:120,186):
        each boundary point takes the value of its inward neighbour at every
        level, one boundary after another."""
        from . import _lib
        from ._pygetm import _p, _s
        import torch

        T = self.T
        t = field.all_values
        fn = "getm_open_boundary_tracers_f32" if t.dtype == torch.float32 else "getm_open_boundary_tracers"
        ptr = _lib.ptr_array([t.data_ptr()])
        for s, e in self.ranges:
            _lib.call(fn, s, e, self.np, T.nx_, T.ny_, t.shape[0], 0, self.i.data_ptr(), self.j.data_ptr(),
                      self.type_zero_gradient.data_ptr(), self.di.data_ptr(), self.dj.data_ptr(), _p(T.mask), 1,
                      ptr, ptr, _s())

    def update_tracers(self, tracers):
        from . import _lib
        from ._pygetm import _p, _s
        import torch

        trs = list(tracers)
        if not trs:
            return
        T = self.T
        f32 = trs[0].all_values.dtype == torch.float32
        fn = "getm_open_boundary_tracers_f32" if f32 else "getm_open_boundary_tracers"
        for c in range(0, len(trs), 16):
            chunk = trs[c:c + 16]
            vars_ = _lib.ptr_array([t.all_values.data_ptr() for t in chunk])
            bdy = _lib.ptr_array([self.tracer_values[t.name].data_ptr() for t in chunk])
            for s, e in self.ranges:
                _lib.call(fn, s, e, self.np, T.nx_, T.ny_, T.nz, self.nsponge, self.i.data_ptr(), self.j.data_ptr(),
                          self.type_3d.data_ptr(), self.di.data_ptr(), self.dj.data_ptr(), _p(T.mask), len(chunk),
                          vars_, bdy, _s())
