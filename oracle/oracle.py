"""CPU oracle for the getm_gb300 CUDA library - TEST INFRASTRUCTURE ONLY.

Python/numpy restatement of pygetm's operator orchestration around the C
restatement of its Fortran kernels (``getm_oracle.c``).  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, as the
reference for comparison; the product path never imports it.

Parity pins: the reference ships no golden vectors and cannot be built here
(no Fortran compiler, empty submodules), so the oracle is pinned by the
known-answer and invariant tests of the reference's own suite
(python/tests/test_vertical_diffusion.py, test_3d_barotropic.py,
test_internal_pressure.py, test_coriolis.py, test_grid.py), ported in
tests/test_oracle_*.py.

Data model: ``OGrid`` holds numpy copies of one staggered grid's static arrays
(from ``getm_gb300.domain.HostGrid``, the shared input set-up) plus the
time-varying depth/thickness fields; arrays are C-ordered [k][j][i] with halos.
"""

from __future__ import annotations

import ctypes
import enum
import functools
from ctypes import c_double, c_int, c_void_p
from typing import Callable, Iterable, Optional

import numpy as np

from . import build as _build

FILL_VALUE = -2e20
RHO0 = 1025.0
GRAVITY = 9.81

import os as _os

# GETM_ORACLE_VARIANT=omp selects the OpenMP build (same results, all cores)
_lib = ctypes.CDLL(str(_build.build(_os.environ.get("GETM_ORACLE_VARIANT", "serial"))))


def load_variant(variant: str):
    return ctypes.CDLL(str(_build.build(variant)))


def _p(a: Optional[np.ndarray], dtype=np.float64):
    if a is None:
        return None
    assert a.dtype == dtype, (a.dtype, dtype)
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(c_void_p)


def _pi(a):
    return _p(a, np.int32)


class AdvectionScheme(enum.IntEnum):
    """python/pygetm/operators.py:11-18"""

    HSIMT = 1
    MUSCL = 2
    P2_PDM = 3
    SPLMAX13 = 4
    SUPERBEE = 5
    UPSTREAM = 6
    DEFAULT = 5


class AdvectionSplit(enum.Enum):
    """python/pygetm/operators.py:21-24"""

    FULL = 1
    HALF = 2
    HALF_ALWAYS = 3


class OGrid:
    """numpy mirror of one staggered grid (static metrics + state)."""

    def __init__(self, hg, nz: Optional[int] = None):
        self.host = hg
        self.nx, self.ny = hg.nx, hg.ny
        self.nz = hg.nz if nz is None else nz
        self.halox, self.haloy = hg.halox, hg.haloy
        self.nx_, self.ny_ = hg.nx_, hg.ny_
        self.imin, self.imax, self.jmin, self.jmax = hg.imin, hg.imax, hg.jmin, hg.jmax
        self.ioffset, self.joffset = hg.ioffset, hg.joffset
        self.postfix = hg.postfix
        for name in ("x", "y", "dx", "dy", "idx", "idy", "area", "iarea", "cor", "H", "z0b_min"):
            setattr(self, name, np.ascontiguousarray(hg.arrays[name], dtype=np.float64).copy())
        self.mask = np.ascontiguousarray(hg.mask, dtype=np.int32).copy()
        self.land = self.mask == 0
        self.water = ~self.land
        self.water_contact = hg.water_contact.copy()
        shape2 = (self.ny_, self.nx_)
        self.D = np.full(shape2, FILL_VALUE)
        self.D[self.water] = self.H[self.water]
        self.z0b = self.z0b_min.copy()
        self.alpha = np.full(shape2, FILL_VALUE)
        nz_ = self.nz
        self.hn = np.full((nz_,) + shape2, FILL_VALUE)
        self.ho = np.full((nz_,) + shape2, FILL_VALUE)
        self.zc = np.broadcast_to(-hg.H_unmasked, (nz_,) + shape2).copy()
        self.zf = np.broadcast_to(-hg.H_unmasked, (nz_ + 1,) + shape2).copy()
        self.ugrid = self.vgrid = self.xgrid = None

    @property
    def interior(self):
        return (Ellipsis, slice(self.haloy, self.haloy + self.ny), slice(self.halox, self.halox + self.nx))


def make_grids(T_host) -> OGrid:
    """Build the OGrid tree mirroring a HostGrid tree (same sharing)."""
    made = {}

    def mk(hg):
        if hg is None:
            return None
        if id(hg) in made:
            return made[id(hg)]
        g = OGrid(hg)
        made[id(hg)] = g
        g.ugrid, g.vgrid, g.xgrid = mk(hg.ugrid), mk(hg.vgrid), mk(hg.xgrid)
        return g

    return mk(T_host)


# ---------------------------------------------------------------------------
# interpolation (python/src/interpolation.F90:9-72 via core.Grid.interpolator,
# python/pygetm/core.py:407-462)
# ---------------------------------------------------------------------------
def interp_x(source, target, offset):
    s = np.ascontiguousarray(source)
    s3 = s if s.ndim == 3 else s[None]
    t3 = target if target.ndim == 3 else target[None]
    _lib.oracle_grid_interp_x(c_int(s3.shape[2]), c_int(s3.shape[1]), c_int(s3.shape[0]), _p(s3), _p(t3), c_int(offset))


def interp_y(source, target, offset):
    s3 = source if source.ndim == 3 else source[None]
    t3 = target if target.ndim == 3 else target[None]
    _lib.oracle_grid_interp_y(c_int(s3.shape[2]), c_int(s3.shape[1]), c_int(s3.shape[0]), _p(s3), _p(t3), c_int(offset))


def interp_z(source, target, offset):
    _lib.oracle_grid_interp_z(c_int(source.shape[2]), c_int(source.shape[1]), c_int(source.shape[0]), c_int(target.shape[0]), _p(source), _p(target), c_int(offset))


def interp_xy(source, target, ioffset, joffset):
    s3 = source if source.ndim == 3 else source[None]
    t3 = target if target.ndim == 3 else target[None]
    _lib.oracle_grid_interp_xy(c_int(s3.shape[2]), c_int(s3.shape[1]), c_int(t3.shape[2]), c_int(t3.shape[1]), c_int(s3.shape[0]), _p(s3), _p(t3), c_int(ioffset), c_int(joffset))


def interpolate(src_grid: OGrid, tgt_grid: OGrid, source, target):
    """core.Grid.interpolator (python/pygetm/core.py:407-462)."""
    a, b = src_grid, tgt_grid
    if a.ioffset == b.ioffset + 1 and a.joffset == b.joffset:
        interp_x(source, target, 1)
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset:
        interp_x(source, target, 0)
    elif a.joffset == b.joffset + 1 and a.ioffset == b.ioffset:
        interp_y(source, target, 1)
    elif a.joffset == b.joffset - 1 and a.ioffset == b.ioffset:
        interp_y(source, target, 0)
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset - 1:
        interp_xy(source, target, 0, 0)
    elif a.ioffset == b.ioffset + 1 and a.joffset == b.joffset + 1:
        interp_xy(source, target, 1, 1)
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset + 1:
        interp_xy(source, target, 0, 1)
    elif a.ioffset == b.ioffset + 1 and a.joffset == b.joffset - 1:
        interp_xy(source, target, 1, 0)
    elif a.ioffset == b.ioffset - 2 and a.joffset == b.joffset:
        target[..., 0:-1] = source[..., 1:]
    elif a.ioffset == b.ioffset and a.joffset == b.joffset - 2:
        target[..., 0:-1, :] = source[..., 1:, :]
    else:
        raise NotImplementedError(f"{a.postfix} -> {b.postfix}")
    return target


# ---------------------------------------------------------------------------
# operators (python/pygetm/operators.py, python/_pygetm.pyx:198-316)
# ---------------------------------------------------------------------------
class Advection:
    """numpy restatement of pygetm.operators.Advection."""

    def __init__(self, grid: OGrid, scheme=AdvectionScheme.DEFAULT, split_2d=AdvectionSplit.HALF):
        self.grid = grid
        self.ugrid, self.vgrid = grid.ugrid, grid.vgrid
        self.scheme = int(scheme)
        self.split_2d = split_2d
        self.ufirst = False
        self.h = np.empty((max(grid.nz, 1), grid.ny_, grid.nx_))
        self.D = self.h[0, ...]
        self.maxiters = 0

    def _uv(self, direction, nk, vel, dt, var, Ah, hvel, h):
        g = self.grid
        vg = self.ugrid if direction == 1 else self.vgrid
        m1, m2 = (vg.idx, vg.dy) if direction == 1 else (vg.dx, vg.idy)
        _lib.oracle_advection_uv_calculate(
            c_int(direction), c_int(nk), c_int(self.scheme), c_int(g.imin), c_int(g.imax), c_int(g.jmin), c_int(g.jmax),
            c_int(g.halox), c_int(g.haloy), _pi(vg.mask), _p(m1), _p(m2), _p(vel), _p(Ah), c_double(dt),
            _p(h), _p(hvel), _p(var), _pi(g.mask), _p(g.iarea),
        )

    # pyx:236-261
    def u_2d(self, u, timestep, var, Ah=None):
        self._uv(1, 1, u, timestep, var, Ah, self.ugrid.D, self.h)

    def v_2d(self, v, timestep, var, Ah=None):
        self._uv(2, 1, v, timestep, var, Ah, self.vgrid.D, self.h)

    def u_3d(self, u, timestep, var, Ah=None):
        self._uv(1, var.shape[0], u, timestep, var, Ah, self.ugrid.hn, self.h)

    def v_3d(self, v, timestep, var, Ah=None):
        self._uv(2, var.shape[0], v, timestep, var, Ah, self.vgrid.hn, self.h)

    def w_3d(self, w, w_var, timestep, var):
        g = self.grid
        it = _lib.oracle_advection_w_calculate(
            c_int(self.scheme), c_int(g.imin), c_int(g.imax), c_int(g.jmin), c_int(g.jmax), c_int(g.nz),
            c_int(g.halox), c_int(g.haloy), _p(w), _p(w_var), _pi(g.mask), c_double(timestep), _p(self.h), _p(var),
        )
        self.maxiters = max(self.maxiters, it)

    def __call__(self, u, v, timestep, var, Ah_u=None, Ah_v=None, skip_initial_halo_exchange=False):
        """operators.py:52-93 (halo exchanges are no-ops on one subdomain)."""
        adv1 = functools.partial(self.u_2d, u, Ah=Ah_u)
        adv2 = functools.partial(self.v_2d, v, Ah=Ah_v)
        if not self.ufirst:
            adv1, adv2 = adv2, adv1
        self.D[...] = self.grid.D
        if self.split_2d == AdvectionSplit.FULL:
            adv1(timestep, var)
            adv2(timestep, var)
        elif self.split_2d == AdvectionSplit.HALF:
            adv1(0.5 * timestep, var)
            adv2(timestep, var)
            adv1(0.5 * timestep, var)
        else:
            adv1(0.5 * timestep, var)
            adv2(0.5 * timestep, var)
            adv2(0.5 * timestep, var)
            adv1(0.5 * timestep, var)

    def apply_3d(self, u, v, w, timestep, var, Ah_u=None, Ah_v=None, new_h=False, skip_initial_halo_exchange=False, w_var=None):
        """operators.py:95-133"""
        if w_var is None:
            w_var = w
        adv1 = functools.partial(self.u_3d, u, 0.5 * timestep, var, Ah_u)
        adv2 = functools.partial(self.v_3d, v, 0.5 * timestep, var, Ah_v)
        if not self.ufirst:
            adv1, adv2 = adv2, adv1
        self.h[...] = self.grid.hn if new_h else self.grid.ho
        adv1()
        adv2()
        self.w_3d(w, w_var, timestep, var)
        adv2()
        adv1()

    def apply_3d_batch(self, u, v, w, timestep, vars: Iterable[np.ndarray], Ah_u=None, Ah_v=None, new_h=False,
                       skip_initial_halo_exchange=False, get_w: Optional[Callable] = None):
        """operators.py:135-193"""
        vars = list(vars)
        if get_w is None:
            get_w = lambda tracer: w  # noqa: E731
        adv1 = functools.partial(self.u_3d, u, 0.5 * timestep, Ah=Ah_u)
        adv2 = functools.partial(self.v_3d, v, 0.5 * timestep, Ah=Ah_v)
        if not self.ufirst:
            adv1, adv2 = adv2, adv1
        current_h = (self.grid.hn if new_h else self.grid.ho).copy()
        for var in vars:
            self.h[...] = current_h
            adv1(var)
        current_h[...] = self.h
        for var in vars:
            self.h[...] = current_h
            adv2(var)
        current_h[...] = self.h
        for var in vars:
            self.h[...] = current_h
            self.w_3d(w, get_w(var), timestep, var)
        current_h[...] = self.h
        for var in vars:
            self.h[...] = current_h
            adv2(var)
        current_h[...] = self.h
        for var in vars:
            self.h[...] = current_h
            adv1(var)


class VerticalAdvection:
    """operators.py:196-215"""

    def __init__(self, grid: OGrid, scheme=AdvectionScheme.DEFAULT):
        self.grid = grid
        self.scheme = int(scheme)
        self.h = np.empty((grid.nz, grid.ny_, grid.nx_))

    def __call__(self, w, w_var, timestep, var, new_h=False):
        self.h[...] = self.grid.hn if new_h else self.grid.ho
        g = self.grid
        _lib.oracle_advection_w_calculate(
            c_int(self.scheme), c_int(g.imin), c_int(g.imax), c_int(g.jmin), c_int(g.jmax), c_int(g.nz),
            c_int(g.halox), c_int(g.haloy), _p(w), _p(w_var), _pi(g.mask), c_double(timestep), _p(self.h), _p(var),
        )


class VerticalDiffusion:
    """pyx:288-316 and operators.py:218-230"""

    def __init__(self, grid: OGrid, cnpar: float = 1.0):
        self.grid = grid
        self.cnpar = cnpar
        shape = (grid.nz, grid.ny_, grid.nx_)
        self.auxo = np.zeros(shape)
        self.auxn = np.zeros(shape)

    def prepare(self, nuh, timestep, molecular=0.0, use_ho=False):
        g = self.grid
        ho = g.ho if use_ho else g.hn
        _lib.oracle_vertical_diffusion_prepare(
            c_int(g.nx_), c_int(g.ny_), c_int(g.nz), c_double(molecular), _p(nuh), c_double(timestep),
            c_double(self.cnpar), _pi(g.mask), _p(ho), _p(g.hn), _p(self.auxo), _p(self.auxn),
        )

    def apply(self, var, ea2=None, ea4=None, use_ho=False):
        g = self.grid
        ho = g.ho if use_ho else g.hn
        _lib.oracle_vertical_diffusion_apply(
            c_int(g.nx_), c_int(g.ny_), c_int(g.nz), _pi(g.mask), _p(ho), _p(g.hn), _p(var), _p(ea2), _p(ea4),
            _p(self.auxo), _p(self.auxn),
        )

    def __call__(self, nuh, timestep, var, molecular=0.0, ea2=None, ea4=None, use_ho=False):
        self.prepare(nuh, timestep, molecular, use_ho)
        self.apply(var, ea2, ea4, use_ho)


# ---------------------------------------------------------------------------
# module functions of _pygetm (pyx:318-572), explicit-array form
# ---------------------------------------------------------------------------
def momentum_diffusion(UG, VG, huu, huv, hvu, hvv, u, v, Am0, diffu, diffv):
    """pyx:318-326 -> wrapper.F90:275-393"""
    UU, UV, VU, VV = UG.ugrid, UG.vgrid, VG.ugrid, VG.vgrid
    nk = u.shape[0] if u.ndim == 3 else 1
    _lib.oracle_momentum_diffusion(
        c_int(UG.nx_), c_int(UG.ny_), c_int(nk), c_int(UG.halox), c_int(UG.haloy),
        _pi(UG.mask), _p(UG.iarea), _pi(VG.mask), _p(VG.iarea),
        _pi(UU.mask), _p(UU.dy), _p(UU.idx),
        _pi(UV.mask), _p(UV.dx), _p(UV.idx), _p(UV.idy),
        _pi(VU.mask), _p(VU.dy), _p(VU.idx), _p(VU.idy),
        _pi(VV.mask), _p(VV.dx), _p(VV.idy),
        _p(huu), _p(huv), _p(hvu), _p(hvv), _p(u), _p(v), c_double(Am0), _p(diffu), _p(diffv),
    )


def thickness2center_depth(g: OGrid, h, out):
    _lib.oracle_thickness2center_depth(c_int(g.nx_), c_int(g.ny_), c_int(h.shape[0]), _pi(g.mask), _p(h), _p(out))


def thickness2vertical_coordinates(g: OGrid, H, h, zc, zf):
    _lib.oracle_thickness2vertical_coordinates(c_int(g.nx_), c_int(g.ny_), c_int(h.shape[0]), _pi(g.mask), _p(H), _p(h), _p(zc), _p(zf))


def alpha(g: OGrid, D, Dmin, Dcrit, out):
    _lib.oracle_alpha(c_int(D.size), _p(D), c_double(Dmin), c_double(Dcrit), _pi(g.mask), _p(out))


def elevation2depth(g: OGrid, z, H, Dmin, D):
    _lib.oracle_elevation2depth(c_int(z.size), _p(z), _p(H), c_double(Dmin), _pi(g.mask), _p(D))


def horizontal_diffusion(g: OGrid, f, Ah_u, Ah_v, dt, out):
    """pyx:369-390"""
    ug, vg = g.ugrid, g.vgrid
    _lib.oracle_horizontal_diffusion(
        c_int(1), c_int(g.nx), c_int(1), c_int(g.ny), c_int(g.halox), c_int(g.haloy),
        _pi(ug.mask), _pi(vg.mask), _p(ug.idx), _p(ug.dy), _p(vg.idy), _p(vg.dx),
        _p(Ah_u), _p(Ah_v), _pi(g.mask), _p(g.iarea), c_double(dt), _p(f), _p(out),
    )


def bottom_friction(g: OGrid, u, v, D, avmmol, out, update_z0b):
    """pyx:392-402"""
    _lib.oracle_bottom_friction(c_int(g.nx_), c_int(g.ny_), _pi(g.mask), _p(u), _p(v), _p(D), _p(g.z0b), _p(g.z0b_min),
                                c_double(avmmol), _p(out), c_int(1 if update_z0b else 0))


def collect_3d_momentum_sources(g: OGrid, dp, cor, adv, diff, idp, taus, rr, dt, ea2, ea4):
    """pyx:404-421"""
    _lib.oracle_collect_3d_momentum_sources(
        c_int(g.nx_), c_int(g.ny_), c_int(g.nz), c_int(g.halox), c_int(g.haloy), _pi(g.mask), _p(g.alpha),
        _p(g.ho), _p(g.hn), _p(dp), _p(cor), _p(adv), _p(diff), _p(idp), _p(taus), _p(rr), c_double(dt), _p(ea2), _p(ea4),
    )


def advance_2d_transport(g: OGrid, U, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r, dt):
    """pyx:423-441"""
    _lib.oracle_advance_2d_transport(
        c_int(g.nx_), c_int(g.ny_), c_int(g.halox), c_int(g.haloy), _pi(g.mask), _p(g.alpha), _p(g.D),
        _p(dp), _p(taus), _p(cor), _p(adv), _p(diff), _p(damp), _p(SA), _p(SB), _p(SD), _p(SF), _p(r), c_double(dt), _p(U),
    )


def w_momentum_3d(T: OGrid, pk, qk, dt, w):
    """pyx:443-455"""
    _lib.oracle_w_momentum_3d(
        c_int(T.nx_), c_int(T.ny_), c_int(T.nz), c_int(T.halox + 1), c_int(T.halox + T.nx + 1),
        c_int(T.haloy + 1), c_int(T.haloy + T.ny + 1), _pi(T.mask), _p(T.ugrid.dy), _p(T.vgrid.dx), _p(T.iarea),
        _p(T.ho), _p(T.hn), _p(pk), _p(qk), c_double(dt), _p(w),
    )


def shear_frequency(T: OGrid, uk, vk, SS):
    """pyx:457-466"""
    _lib.oracle_shear_frequency(
        c_int(T.nx_), c_int(T.ny_), c_int(T.nz), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1),
        c_int(T.haloy + T.ny), _pi(T.mask), _p(T.ugrid.hn), _p(T.vgrid.hn), _p(uk), _p(vk), _p(SS),
    )


def shear_frequency2(T: OGrid, uk, vk, num, SS):
    """pyx:468-479"""
    _lib.oracle_shear_frequency2(
        c_int(T.nx_), c_int(T.ny_), c_int(T.nz), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1),
        c_int(T.haloy + T.ny), _pi(T.mask), _p(T.hn), _p(T.ugrid.hn), _p(T.vgrid.hn), _p(uk), _p(vk), _p(num), _p(SS),
    )


def vertical_advection_to_sources(halox, haloy, mask, c, w, h, s):
    """pyx:574-575 ((nz, ny, nx) arrays; mask int)"""
    nz, ny, nx = c.shape
    _lib.oracle_vertical_advection_to_sources(c_int(nx), c_int(ny), c_int(nz), c_int(halox), c_int(haloy),
                                              _pi(mask), _p(c), _p(w), _p(h), _p(s))


def update_gvc(dsigma, dbeta, Dgamma, kk, D, mask, h):
    """pyx:577-585"""
    nz = dbeta.shape[0]
    ny, nx = D.shape
    if kk < 0:
        kk = nz + kk
    _lib.oracle_update_gvc(c_int(nx), c_int(ny), c_int(nz), c_double(dsigma), _p(np.ascontiguousarray(dbeta)),
                           c_double(Dgamma), c_int(1 + kk), _p(D), _pi(mask), _p(h))


def surface_shear_velocity(T: OGrid, taux, tauy, ustar):
    _lib.oracle_surface_shear_velocity(
        c_int(T.nx_), c_int(T.ny_), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1), c_int(T.haloy + T.ny),
        _pi(T.mask), _p(taux), _p(tauy), _p(ustar),
    )


def bottom_shear_velocity(T: OGrid, uk, vk, rru, rrv, ustar2_x, ustar2_y, ustar):
    """pyx:490-504"""
    _lib.oracle_bottom_shear_velocity(
        c_int(T.nx_), c_int(T.ny_), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1), c_int(T.haloy + T.ny),
        _pi(T.mask), _pi(T.ugrid.mask), _pi(T.vgrid.mask), _p(uk), _p(vk), _p(rru), _p(rrv), _p(ustar2_x), _p(ustar2_y), _p(ustar),
    )


def reconstruct_transport_change(g: OGrid, un, hn, Uo, timestep):
    """pyx:506-510"""
    nz = 1 if Uo.ndim == 2 else g.nz
    _lib.oracle_reconstruct_transport_change(
        c_int(g.nx_), c_int(g.ny_), c_int(nz), c_int(g.halox + 1), c_int(g.halox + g.nx), c_int(g.haloy + 1),
        c_int(g.haloy + g.ny), _p(un), _p(np.ascontiguousarray(hn)), _p(Uo), c_double(timestep),
    )


def advance_surface_elevation(T: OGrid, timestep, z, U, V, fwf):
    """pyx:512-523"""
    _lib.oracle_advance_surface_elevation(
        c_int(T.nx_), c_int(T.ny_), c_int(T.halox), c_int(T.haloy), _pi(T.mask), _p(T.ugrid.dy), _p(T.vgrid.dx),
        _p(T.iarea), _p(z), _p(U), _p(V), _p(fwf), c_double(timestep),
    )


def surface_pressure_gradient(T: OGrid, z, sp, dpdx, dpdy, Dmin):
    """pyx:525-539"""
    U, V = T.ugrid, T.vgrid
    _lib.oracle_surface_pressure_gradient(
        c_int(T.nx_), c_int(T.ny_), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1), c_int(T.haloy + T.ny),
        _pi(U.mask), _pi(V.mask), _p(U.idx), _p(V.idy), _p(z), _p(sp), _p(T.H), _p(T.D), c_double(Dmin), _p(dpdx), _p(dpdy),
    )


def blumberg_mellor(T: OGrid, buoy, idpdx, idpdy):
    """pyx:541-553"""
    U, V = T.ugrid, T.vgrid
    _lib.oracle_blumberg_mellor(
        c_int(T.nx_), c_int(T.ny_), c_int(T.nz), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1),
        c_int(T.haloy + T.ny), _pi(U.mask), _pi(V.mask), _p(U.idx), _p(V.idy), _p(U.hn), _p(V.hn), _p(T.zf),
        _p(buoy), _p(idpdx), _p(idpdy),
    )


def shchepetkin_mcwilliams(T: OGrid, buoy, idpdx, idpdy, zin):
    """pyx:555-568 (z argument is T.zin)"""
    U, V = T.ugrid, T.vgrid
    _lib.oracle_shchepetkin_mcwilliams(
        c_int(T.nx_), c_int(T.ny_), c_int(T.nz), c_int(T.halox + 1), c_int(T.halox + T.nx), c_int(T.haloy + 1),
        c_int(T.haloy + T.ny), _pi(T.mask), _pi(U.mask), _pi(V.mask), _p(U.idx), _p(V.idy), _p(T.hn), _p(zin),
        _p(T.zc), _p(buoy), _p(idpdx), _p(idpdy),
    )


_lib.oracle_advection_w_calculate.restype = c_int
_lib.oracle_limiter.restype = c_double
_lib.oracle_limiter.argtypes = [c_int, c_double, c_double]
