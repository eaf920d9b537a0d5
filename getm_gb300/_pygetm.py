"""GPU counterpart of pygetm's Cython module ``_pygetm`` (python/_pygetm.pyx).

Same function names, argument order and assertions as pyx:180-585; every call
enqueues the matching C-ABI kernel of libgetm_gb300 on the current torch CUDA
stream.  Arguments are ``getm_gb300.core.Array`` objects whose tensors live on
the GPU.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .core import CENTERS, INTERFACES, Array, _sfx, _sfx_storage, interp_x, interp_xy, interp_y, interp_z  # noqa: F401
from ._lib import call


def _s():
    return torch.cuda.current_stream().cuda_stream


def _p(a):
    if a is None:
        return None
    return (a.all_values if isinstance(a, Array) else a).data_ptr()


def momentum_diffusion(huu, huv, hvu, hvv, u, v, Am0, diffu, diffv):
    """pyx:318-326"""
    assert huu.grid is u.grid.ugrid
    assert huv.grid is u.grid.vgrid
    assert hvu.grid is v.grid.ugrid
    assert hvv.grid is v.grid.vgrid
    assert diffu.grid is u.grid
    assert diffv.grid is v.grid
    nk = u.all_values.shape[0] if u.z else 1
    call("getm_momentum_diffusion", u.grid.handle, v.grid.handle, huu.grid.handle, huv.grid.handle, hvu.grid.handle,
         hvv.grid.handle, nk, _p(huu), _p(huv), _p(hvu), _p(hvv), _p(u), _p(v), float(Am0), _p(diffu), _p(diffv), _s())


def thickness2center_depth(mask, h, out=None):
    """pyx:342-348"""
    assert mask.grid is h.grid and h.z == CENTERS
    if out is None:
        out = h.grid.array(z=CENTERS)
    g = mask.grid
    call("getm_thickness2center_depth", g.nx_, g.ny_, g.nz_, 1 + g.halox, g.nx_ - g.halox, 1 + g.haloy, g.ny_ - g.haloy,
         _p(mask), _p(h), _p(out), _s())
    return out


def thickness2vertical_coordinates(mask, H, h, zc, zf):
    """pyx:350-355"""
    assert mask.grid is h.grid and h.z == CENTERS
    assert mask.grid is H.grid and not H.z
    assert mask.grid is zc.grid and zc.z == CENTERS
    assert mask.grid is zf.grid and zf.z == INTERFACES
    g = mask.grid
    call("getm_thickness2vertical_coordinates", g.nx_, g.ny_, g.nz_, _p(mask), _p(H), _p(h), _p(zc), _p(zf), _s())


def alpha(D, Dmin, Dcrit, out):
    """pyx:357-360"""
    call("getm_alpha", D.all_values.numel(), _p(D), float(Dmin), float(Dcrit), _p(D.grid.mask), _p(out), _s())


def elevation2depth(z, H, Dmin, D):
    """pyx:362-367"""
    assert z.grid is H.grid
    assert z.grid is D.grid
    call("getm_elevation2depth", z.all_values.numel(), _p(z), _p(H), float(Dmin), _p(z.grid.mask), _p(D), _s())


def horizontal_diffusion(f, Ah_u, Ah_v, dt, out):
    """pyx:369-390"""
    g = f.grid
    ug, vg = g.ugrid, g.vgrid
    assert not f.z
    assert Ah_u.grid is ug and not Ah_u.z
    assert Ah_v.grid is vg and not Ah_v.z
    assert out.grid is g and not out.z
    call("getm_horizontal_diffusion", 1, g.nx, 1, g.ny, g.halox, g.haloy, _p(ug.mask), _p(vg.mask), _p(ug.idx), _p(ug.dy),
         _p(vg.idy), _p(vg.dx), _p(Ah_u), _p(Ah_v), _p(g.mask), _p(g.iarea), float(dt), _p(f), _p(out), _s())


def bottom_friction(u, v, D, avmmol, out, update_z0b, arithmetic="float64"):
    """pyx:392-402; ``arithmetic="float32"`` evaluates the drag coefficient
    in float (the mixed form), storage stays float64."""
    g = u.grid
    assert not u.z
    assert v.grid is g and not v.z
    assert D.grid is g and not D.z
    assert out.grid is g and not out.z
    fn = "getm_bottom_friction" if arithmetic == "float64" else "getm_bottom_friction_mixed"
    call(fn, g.nx_, g.ny_, _p(g.mask), _p(u), _p(v), _p(D), _p(g.z0b), _p(g.z0b_min), float(avmmol),
         _p(out), 1 if update_z0b else 0, _s())


def collect_3d_momentum_sources(dp, cor, adv, diff, idp, taus, rr, dt, ea2, ea4):
    """pyx:404-421"""
    g = dp.grid
    assert not dp.z, "dp"
    assert cor.grid is g and cor.z == CENTERS, "cor"
    assert adv.grid is g and adv.z == CENTERS, "adv"
    assert diff.grid is g and diff.z == CENTERS, "diff"
    assert idp.grid is g and idp.z == CENTERS, "idp"
    assert taus.grid is g and not taus.z, "taus"
    assert rr.grid is g and not rr.z, "rr"
    assert ea2.z == CENTERS
    assert ea4.z == CENTERS
    sfx = _sfx(cor.all_values, adv.all_values, diff.all_values, ea2.all_values, ea4.all_values)
    if idp.all_values.dtype != torch.float64:
        raise TypeError("the internal pressure gradient idp must be float64 in both forms")
    call("getm_collect_3d_momentum_sources" + sfx, g.nx_, g.ny_, g.nz, g.halox, g.haloy, _p(g.mask), _p(g.alpha), _p(g.ho),
         _p(g.hn), _p(dp), _p(cor), _p(adv), _p(diff), _p(idp), _p(taus), _p(rr), float(dt), _p(ea2), _p(ea4), _s())


def advance_2d_transport(U, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r, dt, mixed=False):
    """pyx:423-441; ``mixed``: tendency in float, transport update in double."""
    g = U.grid
    for a, n in ((dp, "dp"), (taus, "taus"), (cor, "cor"), (adv, "adv"), (diff, "diff"), (damp, "damp"), (SA, "SA"),
                 (SB, "SB"), (SD, "SD"), (SF, "SF"), (r, "rr")):
        assert a.grid is g and not a.z, n
    call("getm_advance_2d_transport_mixed" if mixed else "getm_advance_2d_transport", g.nx_, g.ny_, g.halox, g.haloy, _p(g.mask), _p(g.alpha), _p(g.D), _p(dp), _p(taus),
         _p(cor), _p(adv), _p(diff), _p(damp), _p(SA), _p(SB), _p(SD), _p(SF), _p(r), float(dt), _p(U), _s())


def w_momentum_3d(pk, qk, dt, w):
    """pyx:443-455"""
    g = w.grid
    assert w.z == INTERFACES, "w"
    assert pk.grid is g.ugrid and pk.z == CENTERS, "pk"
    assert qk.grid is g.vgrid and qk.z == CENTERS, "qk"
    call("getm_w_momentum_3d" + _sfx(pk.all_values, qk.all_values, w.all_values), g.nx_, g.ny_, g.nz, g.halox + 1, g.halox + g.nx + 1, g.haloy + 1, g.haloy + g.ny + 1,
         _p(g.mask), _p(pk.grid.dy), _p(qk.grid.dx), _p(g.iarea), _p(g.ho), _p(g.hn), _p(pk), _p(qk), float(dt), _p(w), _s())


def shear_frequency(uk, vk, SS):
    """pyx:457-466"""
    g = SS.grid
    assert SS.z == INTERFACES, "w"
    assert uk.grid is g.ugrid and uk.z == CENTERS, "uk"
    assert vk.grid is g.vgrid and vk.z == CENTERS, "vk"
    call("getm_shear_frequency" + _sfx(uk.all_values, vk.all_values, SS.all_values), g.nx_, g.ny_, g.nz, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(g.mask), _p(uk.grid.hn), _p(vk.grid.hn), _p(uk), _p(vk), _p(SS), _s())


def shear_frequency2(uk, vk, num, SS):
    """pyx:468-479"""
    g = SS.grid
    assert SS.z == INTERFACES, "w"
    assert uk.grid is g.ugrid and uk.z == CENTERS, "uk"
    assert vk.grid is g.vgrid and vk.z == CENTERS, "vk"
    assert num.grid is g and num.z == INTERFACES, "num"
    sfx = _sfx(uk.all_values, vk.all_values, num.all_values, SS.all_values)
    call("getm_shear_frequency2" + sfx, g.nx_, g.ny_, g.nz, g.halox + 1, g.halox + g.nx, g.haloy + 1,
         g.haloy + g.ny, _p(g.mask), _p(g.hn), _p(uk.grid.hn), _p(vk.grid.hn), _p(uk), _p(vk), _p(num), _p(SS), _s())


def surface_shear_velocity(taux, tauy, ustar):
    """pyx:481-488"""
    g = ustar.grid
    assert not ustar.z, "ustar"
    assert taux.grid is g and not taux.z, "taux"
    assert tauy.grid is g and not tauy.z, "tauy"
    call("getm_surface_shear_velocity", g.nx_, g.ny_, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(g.mask), _p(taux), _p(tauy), _p(ustar), _s())


def bottom_shear_velocity(uk, vk, rru, rrv, ustar2_x, ustar2_y, ustar):
    """pyx:490-504"""
    g = ustar.grid
    assert not ustar.z, "ustar"
    assert uk.grid is g.ugrid, "uk"
    assert vk.grid is g.vgrid, "vk"
    assert rru.grid is g.ugrid and not rru.z, "rru"
    assert rrv.grid is g.vgrid and not rrv.z, "rrv"
    assert ustar2_x.grid is g.ugrid and not ustar2_x.z, "ustar2_x"
    assert ustar2_y.grid is g.vgrid and not ustar2_y.z, "ustar2_y"
    call("getm_bottom_shear_velocity", g.nx_, g.ny_, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(g.mask), _p(g.ugrid.mask), _p(g.vgrid.mask), _p(uk), _p(vk), _p(rru), _p(rrv), _p(ustar2_x),
         _p(ustar2_y), _p(ustar), _s())


def reconstruct_transport_change(un, hn, Uo, timestep):
    """pyx:506-510 (hn is a raw tensor, like the reference's ndarray)"""
    g = Uo.grid
    nz = 1 if Uo.ndim == 2 else g.nz_
    call("getm_reconstruct_transport_change" + _sfx(un.all_values, Uo.all_values), g.nx_, g.ny_, nz, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(un), _p(hn), _p(Uo), float(timestep), _s())


def advance_surface_elevation(timestep, z, U, V, fwf):
    """pyx:512-523"""
    g = z.grid
    assert not z.z, "z"
    assert U.grid is g.ugrid and not U.z, "U"
    assert V.grid is g.vgrid and not V.z, "V"
    assert fwf.grid is g and not fwf.z, "fwf"
    call("getm_advance_surface_elevation", g.nx_, g.ny_, g.halox, g.haloy, _p(g.mask), _p(U.grid.dy), _p(V.grid.dx),
         _p(g.iarea), _p(z), _p(U), _p(V), _p(fwf), float(timestep), _s())


def surface_pressure_gradient(z, sp, dpdx, dpdy, Dmin, mixed=False):
    """pyx:525-539 (mixed: the mixed-form arithmetic, getm_surface_pressure_gradient_mixed)"""
    g = z.grid
    assert not z.z, "z"
    assert sp.grid is g and not sp.z, "sp"
    assert dpdx.grid is g.ugrid and not dpdx.z, "dpdx"
    assert dpdy.grid is g.vgrid and not dpdy.z, "dpdy"
    fn = "getm_surface_pressure_gradient_mixed" if mixed else "getm_surface_pressure_gradient"
    call(fn, g.nx_, g.ny_, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(dpdx.grid.mask), _p(dpdy.grid.mask), _p(dpdx.grid.idx), _p(dpdy.grid.idy), _p(z), _p(sp), _p(g.H), _p(g.D),
         float(Dmin), _p(dpdx), _p(dpdy), _s())


def blumberg_mellor(buoy, idpdx, idpdy):
    """pyx:541-553"""
    g = buoy.grid
    assert buoy.z == CENTERS, "buoy"
    assert idpdx.grid is g.ugrid and idpdx.z == CENTERS, "idpdx"
    assert idpdy.grid is g.vgrid and idpdy.z == CENTERS, "idpdy"
    call("getm_blumberg_mellor" + _sfx(buoy.all_values, idpdx.all_values, idpdy.all_values), g.nx_, g.ny_, g.nz_, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(idpdx.grid.mask), _p(idpdy.grid.mask), _p(idpdx.grid.idx), _p(idpdy.grid.idy), _p(idpdx.grid.hn),
         _p(idpdy.grid.hn), _p(g.zf), _p(buoy), _p(idpdx), _p(idpdy), _s())


_P_WORK = {}


def shchepetkin_mcwilliams(buoy, idpdx, idpdy, P_work=None, arithmetic="float64"):
    """pyx:555-568.  ``P_work`` (optional) is the 3D pressure work array (nz
    planes, nz + 2 for ``arithmetic="float32"``); by default one per grid is
    kept.  ``arithmetic="float32"`` (float64 fields)
    evaluates the slope corrections in float (the mixed form)."""
    g = buoy.grid
    assert buoy.z == CENTERS, "buoy"
    assert idpdx.grid is g.ugrid and idpdx.z == CENTERS, "idpdx"
    assert idpdy.grid is g.vgrid and idpdy.z == CENTERS, "idpdy"
    nz, ny, nx = buoy.all_values.shape
    shape = (nz + 2, ny, nx)  # the mixed form keeps two planes of column terms after P
    if P_work is None:
        P_work = _P_WORK.get(id(g))
        if P_work is None or P_work.shape != shape:
            P_work = torch.zeros(shape, dtype=torch.float64, device=buoy.all_values.device)
            _P_WORK[id(g)] = P_work
    assert P_work.shape[1:] == (ny, nx) and P_work.shape[0] >= nz and P_work.dtype == torch.float64
    if arithmetic == "float32":
        assert P_work.shape[0] >= nz + 2, "P_work: nz + 2 planes for the mixed form"
    sfx = _sfx(buoy.all_values, idpdx.all_values, idpdy.all_values)
    if arithmetic == "float32" and sfx == "":
        sfx = "_mixed"
    call("getm_shchepetkin_mcwilliams" + sfx, g.nx_, g.ny_, g.nz_, g.halox + 1, g.halox + g.nx, g.haloy + 1, g.haloy + g.ny,
         _p(g.mask), _p(idpdx.grid.mask), _p(idpdy.grid.mask), _p(idpdx.grid.idx), _p(idpdy.grid.idy), _p(g.hn),
         _p(g.zin), _p(g.zc), _p(buoy), _p(idpdx), _p(idpdy), P_work.data_ptr(), _s())


def multiply_add(tgt: torch.Tensor, add: torch.Tensor, scale_factor: float):
    """pyx:570-572"""
    if tgt.numel() != 0:
        call("getm_multiply_add", tgt.numel(), tgt.data_ptr(), add.data_ptr(), float(scale_factor), _s())


_flags = {}


def vertical_advection_to_sources(halox: int, haloy: int, mask: torch.Tensor, c: torch.Tensor, w: torch.Tensor,
                                  h: torch.Tensor, s: torch.Tensor):
    """pyx:574-575: (nz, ny, nx) device tensors, mask int32, the rest float64."""
    nz, ny, nx = c.shape
    for name, t, dt in (("mask", mask, torch.int32), ("w", w, torch.float64), ("h", h, torch.float64),
                        ("s", s, torch.float64), ("c", c, torch.float64)):
        assert t.shape == (nz, ny, nx) and t.dtype == dt and t.is_contiguous(), name
    flag = _flags.get(c.device)
    if flag is None:
        flag = _flags[c.device] = torch.zeros(1, dtype=torch.int32, device=c.device)
    call("getm_vertical_advection_to_sources", nx, ny, nz, halox, haloy, mask.data_ptr(), c.data_ptr(), w.data_ptr(),
         h.data_ptr(), s.data_ptr(), flag.data_ptr(), _s())


def update_gvc(dsigma: float, dbeta: torch.Tensor, Dgamma: float, kk: int, D: torch.Tensor, mask: torch.Tensor,
               h: torch.Tensor):
    """pyx:577-585: dbeta (nz,), D (ny, nx) float64 and mask (ny, nx) int32
    device tensors; h (nz, ny, nx) float64; kk < 0 counts from the top."""
    ny, nx = D.shape
    nz = dbeta.shape[0]
    assert mask.shape == (ny, nx) and mask.dtype == torch.int32
    assert h.shape == (nz, ny, nx) and h.dtype == torch.float64 and h.is_contiguous()
    assert D.dtype == torch.float64 and dbeta.dtype == torch.float64
    if kk < 0:
        kk = nz + kk
    call("getm_update_gvc", nx, ny, nz, float(dsigma), dbeta.data_ptr(), float(Dgamma), 1 + kk, D.data_ptr(),
         mask.data_ptr(), h.data_ptr(), _s())


def new_handle():
    return ctypes.c_void_p()


# ---------------------------------------------------------------------------
# fused sequences of the 2D substep (no single counterpart in the reference;
# each replaces the operations named in its docstring with one launch)
# ---------------------------------------------------------------------------
def update_depth_2d(T, z, zo, Dmin, Dcrit, mixed=False):
    """Simulation.update_depth, 2D part (simulation.py:1498-1586):
    elevation2depth on T, Dclip, z_T_half and its interpolation to U, V, X,
    depths and alpha there, D_T_half and the UU/VV/UV/VU depth copies
    (mixed: alpha in float, getm_update_depth_2d_mixed)."""
    U, V, X = T.ugrid, T.vgrid, T.xgrid
    fn = "getm_update_depth_2d_mixed" if mixed else "getm_update_depth_2d"
    call(fn, T.nx_, T.ny_, float(Dmin), float(Dcrit), _p(z), _p(zo), _p(T.H), _p(U.H), _p(V.H),
         _p(X.H), _p(T.mask), _p(U.mask), _p(V.mask), _p(X.mask), _p(T.D), _p(T.Dclip), _p(T._work), _p(U._work),
         _p(U.D), _p(U.alpha), _p(V._work), _p(V.D), _p(V.alpha), _p(X._work), _p(X.D), _p(U.ugrid.D),
         _p(V.vgrid.D), _p(U.vgrid.D), _p(V.ugrid.D), _s())


def momentum_2d_velocities(U, V, u1, v1, advU, advV, uua, uva, vua, vva, mixed=False):
    """momentum.py:1017-1040 (Am = 0 part): u1 = U/D, v1 = V/D, the advected
    copies and the advection velocities on the UU, UV, VU, VV grids."""
    g = U.grid
    call("getm_momentum_2d_velocities", g.nx_, g.ny_, int(bool(mixed)), _p(U), _p(V), _p(U.grid.D), _p(V.grid.D),
         _p(uua.grid.D), _p(uva.grid.D), _p(vua.grid.D), _p(vva.grid.D), _p(u1), _p(v1), _p(advU), _p(advV),
         _p(uua), _p(uva), _p(vua), _p(vva), _s())


def momentum_2d_friction(u1, v1, ru, rv, mixed=False):
    """Momentum.bottom_friction on the U and V grids (momentum.py:1099-1125,
    momentum.F90:79-101 without z0b iteration)."""
    ug, vg = u1.grid, v1.grid
    call("getm_momentum_2d_friction", ug.nx_, ug.ny_, int(bool(mixed)), _p(ug.mask), _p(vg.mask), _p(u1), _p(v1),
         _p(ug.D), _p(vg.D), _p(ug.z0b), _p(vg.z0b), _p(ug._work), _p(vg._work), _p(ru), _p(rv), _s())


def coriolis_2d(U, out, x_direction, mixed=False):
    """Momentum.coriolis, DEFAULT scheme, for 2D transports (momentum.py:1127-1148);
    ``mixed``: in float arithmetic."""
    a, b = U.grid, out.grid
    if a.ioffset == b.ioffset + 1 and a.joffset == b.joffset - 1:
        io, jo = 1, 0
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset + 1:
        io, jo = 0, 1
    else:
        raise NotImplementedError("coriolis_2d expects U -> V or V -> U")
    call("getm_coriolis_2d_mixed" if mixed else "getm_coriolis_2d", b.nx_, b.ny_, io, jo, _p(U), _p(b.cor), _p(out),
         int(bool(x_direction)), _s())


def coriolis_3d(U, out, x_direction):
    """Momentum.coriolis, DEFAULT scheme, for 3D transports (momentum.py:1127-1148)."""
    a, b = U.grid, out.grid
    if a.ioffset == b.ioffset + 1 and a.joffset == b.joffset - 1:
        io, jo = 1, 0
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset + 1:
        io, jo = 0, 1
    else:
        raise NotImplementedError("coriolis_3d expects U -> V or V -> U")
    sfx = _sfx(U.all_values, out.all_values)
    call("getm_coriolis_3d" + sfx, b.nx_, b.ny_, out.all_values.shape[0], io, jo, _p(U), _p(b.cor), _p(out),
         int(bool(x_direction)), _s())


def coriolis_espelid(U, out, x_direction):
    """Momentum.coriolis, ESPELID scheme (momentum.py:1136-1142), for 2D or 3D
    transports: f * sqrt(Dout) * interp(U / sqrt(Din)), negated for the V
    equation, with D the water depths (2D) or layer thicknesses (3D)."""
    a, b = U.grid, out.grid
    if a.ioffset == b.ioffset + 1 and a.joffset == b.joffset - 1:
        io, jo = 1, 0
    elif a.ioffset == b.ioffset - 1 and a.joffset == b.joffset + 1:
        io, jo = 0, 1
    else:
        raise NotImplementedError("coriolis_espelid expects U -> V or V -> U")
    if U.z:
        Din, Dout, nz = a.hn, b.hn, out.all_values.shape[0]
    else:
        Din, Dout, nz = a.D, b.D, 1
    sfx = _sfx(U.all_values, out.all_values)
    call("getm_coriolis_espelid" + sfx, b.nx_, b.ny_, nz, io, jo, _p(U), _p(Din), _p(a.mask), _p(Dout), _p(b.mask),
         _p(b.cor), _p(out), int(bool(x_direction)), _s())


def accumulate_2d(U, V, Ucum, Vcum):
    """_U_cum += U; _V_cum += V (momentum.py:716-718)."""
    call("getm_accumulate_2d", U.all_values.numel(), _p(U), _p(V), Ucum.data_ptr(), Vcum.data_ptr(), _s())


def surface_elevation_fused(timestep, z, zo, U, V, fwf):
    """zo = z, then advance_surface_elevation (simulation.py:1468-1486)."""
    g = z.grid
    call("getm_surface_elevation_fused", g.nx_, g.ny_, g.halox, g.haloy, _p(g.mask), _p(U.grid.dy), _p(V.grid.dx),
         _p(g.iarea), _p(z), _p(zo), _p(U), _p(V), _p(fwf), float(timestep), _s())


# ---- one 2D substep as one launch -----------------------------------------
# field order of getm_split2d_fields (include/getm_gb300.h); every member is
# a device pointer
SPLIT2D_FIELDS = (
    "mask_t", "H_t", "iarea_t", "z", "zo", "D_t", "Dclip_t", "work_t", "fwf", "pe", "sp", "taux", "tauy",
    "mask_u", "H_u", "dy_u", "idx_u", "cor_u", "z0b_u", "D_u", "alpha_u", "work_u",
    "U", "dpdx", "tausx", "corU", "advU", "diffU", "dampU", "SxA", "SxB", "SxD", "SxF",
    "ru", "u1", "Ucum", "advD_u", "uua", "uva",
    "mask_v", "H_v", "dx_v", "idy_v", "cor_v", "z0b_v", "D_v", "alpha_v", "work_v",
    "V", "dpdy", "tausy", "corV", "advV", "diffV", "dampV", "SyA", "SyB", "SyD", "SyF",
    "rv", "v1", "Vcum", "advD_v", "vua", "vva",
    "mask_x", "H_x", "D_x", "work_x", "D_uu", "D_uv", "D_vu", "D_vv", "time", "sync",
)


class Split2DFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in SPLIT2D_FIELDS]


def split2d_fields(**arrays) -> Split2DFields:
    """The fields struct from Arrays or tensors (every name of SPLIT2D_FIELDS;
    ``time`` may be None)."""
    missing = set(SPLIT2D_FIELDS) - set(arrays) - {"time"}
    if missing:
        raise ValueError(f"split2d_fields: missing {sorted(missing)}")
    f = Split2DFields()
    for n in SPLIT2D_FIELDS:
        a = arrays.get(n)
        setattr(f, n, None if a is None else (a.data_ptr() if isinstance(a, torch.Tensor) else _p(a)))
    return f


def split2d_substep(fields: Split2DFields, T, mixed, ufirst, accumulate, friction, timestep, Dmin, Dcrit, uadv, vadv):
    """One non-macro 2D substep (simulation.py:1033-1304 with update_3d
    false) as one launch; ``uadv``/``vadv``: the momentum Advection objects."""
    U, V = T.ugrid, T.vgrid
    call("getm_split2d_substep", ctypes.byref(fields), T.nx_, T.ny_, T.halox, T.haloy, int(bool(mixed)),
         int(bool(ufirst)), int(bool(accumulate)), int(bool(friction)), float(timestep), float(Dmin), float(Dcrit),
         uadv.p, U.handle, U.ugrid.handle, U.vgrid.handle, int(uadv.ufirst),
         vadv.p, V.handle, V.ugrid.handle, V.vgrid.handle, int(vadv.ufirst), _s())


def transport_3d_finish(vel3d, hn, tp2d, D, tp3d, dev):
    """Momentum.advance_3d_transport after the vertical diffusion
    (momentum.py:1199-1210): tp3d = vel3d hn, dev = (sum_k tp3d - tp2d) / D,
    tp3d -= dev hn."""
    g = tp3d.grid
    sfx = _sfx(vel3d.all_values, tp3d.all_values)
    call("getm_transport_3d_finish" + sfx, g.nx_, g.ny_, tp3d.all_values.shape[0], _p(vel3d), _p(hn), _p(tp2d), _p(D),
         _p(tp3d), _p(dev), _s())


def velocities_3d(pk, qk, uk, vk, ubot=None, vbot=None):
    """uk = pk / hn_U, vk = qk / hn_V (momentum.py:909-910); with ``ubot``,
    ``vbot`` (mixed form) also their bottom layers widened to FP64."""
    sfx = _sfx(pk.all_values, qk.all_values, uk.all_values, vk.all_values)
    if ubot is not None:
        if sfx != "_f32":
            raise TypeError("bottom velocities are written by the float form only")
        call("getm_velocities_3d_bottom_f32", pk.all_values.numel(), ubot.all_values.numel(), _p(pk),
             _p(pk.grid.hn), _p(qk), _p(qk.grid.hn), _p(uk), _p(vk), _p(ubot), _p(vbot), _s())
        return
    call("getm_velocities_3d" + sfx, pk.all_values.numel(), _p(pk), _p(pk.grid.hn), _p(qk), _p(qk.grid.hn), _p(uk),
         _p(vk), _s())


def mean_transports(Ucum, Vcum, scale, Ui, Vi):
    """Ui = U_cum scale, Vi = V_cum scale, then U_cum = V_cum = 0
    (momentum.py:790-793); U_cum, V_cum are tensors."""
    call("getm_mean_transports", Ucum.numel(), Ucum.data_ptr(), Vcum.data_ptr(), float(scale), _p(Ui), _p(Vi), _s())


def slow_friction(ustar2x, ru, u1, SxF, ustar2y, rv, v1, SyF):
    """SxF = ustar2_bx + ru u1, SyF = ustar2_by + rv v1 (momentum.py:1003-1015)."""
    call("getm_slow_friction", SxF.all_values.numel(), _p(ustar2x), _p(ru), _p(u1), _p(SxF), _p(ustar2y), _p(rv),
         _p(v1), _p(SyF), _s())


# field order of getm_depth3d_fields (include/getm_gb300.h)
DEPTH3D_FIELDS = (
    "dga", "mask_t", "mask_u", "mask_v", "mask_x", "Dclip_t", "Dclip_u", "Dclip_v", "Dclip_x", "H_t", "H_u", "H_v",
    "hn_t", "hn_u", "hn_v", "hn_x", "ho_t", "ho_u", "ho_v", "zc_t", "zc_u", "zc_v", "zf_t", "zf_u", "zf_v", "depth",
    "h_T_half", "hn_uu", "hn_vv", "hn_uv", "hn_vu",
)


class Depth3DFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in DEPTH3D_FIELDS]


def depth3d_fields(T, dga, h_T_half, depth=None) -> Depth3DFields:
    """Fields of getm_update_depth_3d for the grid tree of T (``depth``: the
    T centre depths, or None)."""
    U, V, X = T.ugrid, T.vgrid, T.xgrid
    assert dga.is_contiguous() and dga.dtype == torch.float64
    arrays = dict(dga=dga, mask_t=T.mask, mask_u=U.mask, mask_v=V.mask, mask_x=X.mask, Dclip_t=T.Dclip,
                  Dclip_u=U.Dclip, Dclip_v=V.Dclip, Dclip_x=X.Dclip, H_t=T.H, H_u=U.H, H_v=V.H, hn_t=T.hn, hn_u=U.hn,
                  hn_v=V.hn, hn_x=X.hn, ho_t=T.ho, ho_u=U.ho, ho_v=V.ho, zc_t=T.zc, zc_u=U.zc, zc_v=V.zc, zf_t=T.zf,
                  zf_u=U.zf, zf_v=V.zf, depth=depth, h_T_half=h_T_half, hn_uu=U.ugrid.hn, hn_vv=V.vgrid.hn,
                  hn_uv=U.vgrid.hn, hn_vu=V.ugrid.hn)
    f = Depth3DFields()
    for n in DEPTH3D_FIELDS:
        a = arrays[n]
        setattr(f, n, None if a is None else (a.data_ptr() if isinstance(a, torch.Tensor) else _p(a)))
    return f


def update_depth_3d(fields: Depth3DFields, T):
    """Simulation.update_depth, 3D part (simulation.py:1588-1630)."""
    call("getm_update_depth_3d", ctypes.byref(fields), T.nx_, T.ny_, T.nz_, _s())


def column_sums(pairs, subtract=False):
    """dst = sum_k src (minus the old dst with ``subtract``) for up to four
    (src 3D Array, dst 2D Array) pairs on grids of the same extents
    (momentum.py:989-1012, simulation.py:1186-1192)."""
    assert 1 <= len(pairs) <= 4
    src0 = pairs[0][0]
    g = src0.grid
    args = []
    for s, d in pairs:
        assert d.all_values.dtype == torch.float64 and s.all_values.shape[1:] == d.all_values.shape
        args += [_p(s), _p(d)]
    args += [None, None] * (4 - len(pairs))
    sfx = _sfx(*[s.all_values for s, _ in pairs])
    call("getm_column_sums" + sfx, g.nx_, g.ny_, src0.all_values.shape[0], int(bool(subtract)), *args, _s())


def buoyancy_frequency(salt, temp, p, out):
    """Density.get_buoyancy_frequency (density.py:22-60) for the device EOS:
    squared buoyancy frequency at the interior interfaces of ``out``
    (z=INTERFACES); ``p``: layer-centre depths (thickness2center_depth)."""
    g = salt.grid
    assert temp.grid is g and p.grid is g and out.grid is g and out.z == INTERFACES
    sfx = _sfx_storage([out.all_values], [salt.all_values, temp.all_values])
    call("getm_buoyancy_frequency" + sfx, g.nx_, g.ny_, salt.all_values.shape[0], _p(g.mask), _p(g.hn), _p(p),
         _p(salt), _p(temp), _p(out), _s())
    return out


def momentum_3d_advection_inputs(uk, vk, ww, uua, uva, vua, vva, wwu, wwv, advpk, advqk):
    """The interpolated velocities and advected copies of the 3D momentum
    advection (momentum.py:989-1003) in one launch."""
    U, V, T = uk.grid, vk.grid, ww.grid
    assert uua.grid is U.ugrid and uva.grid is U.vgrid and vua.grid is V.ugrid and vva.grid is V.vgrid
    assert wwu.grid is U and wwv.grid is V and ww.z == INTERFACES
    # the interpolations these grids imply (core.Grid.interpolate): +1 in i -> interp_x, +1 in j -> interp_y
    for s, d, di, dj in ((U, U.ugrid, 1, 0), (V, U.vgrid, 1, 0), (U, V.ugrid, 0, 1), (V, V.vgrid, 0, 1),
                         (T, U, 1, 0), (T, V, 0, 1)):
        assert d.ioffset - s.ioffset == di and d.joffset - s.joffset == dj
    sfx = _sfx(uk.all_values, vk.all_values, ww.all_values)
    call("getm_momentum_3d_advection_inputs" + sfx, T.nx_, T.ny_, uk.all_values.shape[0], _p(uk), _p(vk), _p(ww),
         _p(uua), _p(uva), _p(vua), _p(vva), _p(wwu), _p(wwv), _p(advpk), _p(advqk), _s())
