"""2D and 3D momentum on the GPU: counterpart of pygetm.momentum.Momentum
(python/pygetm/momentum.py:24-1214) for closed domains.

Field names, the order of operations and the Coriolis/advection/friction
coupling follow the reference; every kernel is a libgetm_gb300 launch (via
``_pygetm``/``operators``) or a torch elementwise op on device tensors.
"""

from __future__ import annotations

import enum
from typing import Optional

import torch

from . import _pygetm
from .core import CENTERS, INTERFACES, Array, Grid
from .domain import FILL_VALUE
from .operators import Advection, AdvectionScheme, AdvectionSplit, VerticalDiffusion


class CoriolisScheme(enum.IntEnum):
    """python/pygetm/momentum.py:14-17"""

    OFF = 0
    DEFAULT = 1
    ESPELID = 2


MASK_ZERO_2D = ("U", "V", "u1", "v1")  # momentum.py:20
MASK_ZERO_3D = ("pk", "qk", "uk", "vk", "Ui", "Vi", "rru", "rrv")  # momentum.py:21


class Momentum:
    def __init__(self, Am: float = 0.0, An: float = 0.0, cnpar: float = 1.0,
                 advection_scheme: Optional[AdvectionScheme] = None,
                 advection_split_2d: AdvectionSplit = AdvectionSplit.FULL,
                 coriolis_scheme: CoriolisScheme = CoriolisScheme.DEFAULT, avmmol: float = 1.8e-6,
                 dtype: torch.dtype = torch.float64):
        """momentum.py:113-144.  ``dtype`` is the type of the 3D (depth-explicit)
        fields: float64 for the FP64 form, float32 for the mixed form; 2D
        transports and everything tied to layer thickness stay float64."""
        self._Am_const = Am
        self._An_const = An
        self.cnpar = cnpar
        self.advection_scheme = advection_scheme
        self.advection_split_2d = advection_split_2d
        self.coriolis_scheme = coriolis_scheme
        self.avmmol = avmmol
        self.dtype3d = dtype
        # fused 2D substep kernels (one launch per sequence of operations);
        # False runs each operation as its own kernel
        self.fused_2d = True
        self._v_stream = None  # see _diagnostics_tail
        self._bottom_event = torch.cuda.Event() if torch.cuda.is_available() else None
        self._ob = None  # open-boundary operations (set by the simulation)

    # ------------------------------------------------------------------ setup
    def _create_arrays(self, tgrid: Grid, three_d: bool):
        """momentum.py:146-487 (fill values as in the reference)."""
        ug, vg = tgrid.ugrid, tgrid.vgrid
        for n in ("U", "u1", "SxA", "SxB", "SxD", "SxF", "corU", "advU", "diffU", "dampU", "ru"):
            setattr(self, n, ug.array(name=n))
        for n in ("V", "v1", "SyA", "SyB", "SyD", "SyF", "corV", "advV", "diffV", "dampV", "rv"):
            setattr(self, n, vg.array(name=n))
        nan = float("nan")
        self.uua = ug.ugrid.array(fill=nan)
        self.uva = ug.vgrid.array(fill=nan)
        self.vua = vg.ugrid.array(fill=nan)
        self.vva = vg.vgrid.array(fill=nan)
        if not three_d:
            return
        d3 = self.dtype3d
        for n in ("pk", "uk", "corpk", "advpk", "diffpk"):
            setattr(self, n, ug.array(name=n, z=CENTERS, dtype=d3))
        for n in ("qk", "vk", "corqk", "advqk", "diffqk"):
            setattr(self, n, vg.array(name=n, z=CENTERS, dtype=d3))
        self.ww = tgrid.array(name="ww", z=INTERFACES, dtype=d3)
        self.SS = tgrid.array(name="SS", z=INTERFACES, dtype=d3)
        for n in ("rru", "Ui", "udev", "ustar2_bx"):
            setattr(self, n, ug.array(name=n))
        for n in ("rrv", "Vi", "vdev", "ustar2_by"):
            setattr(self, n, vg.array(name=n))
        self._U_cum = torch.zeros_like(self.Ui.all_values)
        self._V_cum = torch.zeros_like(self.Vi.all_values)
        self.uua3d = ug.ugrid.array(fill=nan, z=CENTERS, dtype=d3)
        self.uva3d = ug.vgrid.array(fill=nan, z=CENTERS, dtype=d3)
        self.vua3d = vg.ugrid.array(fill=nan, z=CENTERS, dtype=d3)
        self.vva3d = vg.vgrid.array(fill=nan, z=CENTERS, dtype=d3)
        self.ustar_b = tgrid.array(name="ustar_b")
        # interpolation targets reused every step (pygetm allocates these per call)
        self._visc_u = ug.array(z=INTERFACES, fill_value=None, dtype=d3)
        self._visc_v = vg.array(z=INTERFACES, fill_value=None, dtype=d3)
        self._ww_u = ug.array(z=INTERFACES, fill_value=None, dtype=d3)
        self._ww_v = vg.array(z=INTERFACES, fill_value=None, dtype=d3)
        # bottom-layer velocities for the FP64 2D friction kernels
        self._u_bot64 = ug.array(fill=0.0)
        self._v_bot64 = vg.array(fill=0.0)

    def initialize(self, tgrid: Grid, runtype: int, default_advection_scheme: AdvectionScheme):
        """momentum.py:489-616"""
        three_d = runtype > 1
        self._create_arrays(tgrid, three_d)
        ug, vg = tgrid.ugrid, tgrid.vgrid
        self.runtype = runtype
        z0b_u = (ug.z0b_min.all_values[ug.water] == 0.0).any()
        z0b_v = (vg.z0b_min.all_values[vg.water] == 0.0).any()
        self.apply_bottom_friction = not bool(z0b_u or z0b_v)
        self.diffuse_momentum = self._Am_const > 0.0
        zero_everywhere = MASK_ZERO_2D + (MASK_ZERO_3D if three_d else ())
        zero_unmasked = ("SxA", "SyA", "SxB", "SyB", "SxD", "SyD", "SxF", "SyF", "dampU", "dampV", "advU", "advV",
                         "diffU", "diffV", "ru", "rv", "corU", "corV")
        if three_d:
            zero_unmasked += ("SS", "advpk", "advqk", "diffpk", "diffqk", "corpk", "corqk", "ww")
        for n in zero_everywhere:
            getattr(self, n).all_values.zero_()
        for n in zero_unmasked:
            getattr(self, n).fill(0.0)
        self.corU.all_values[:, -1] = 0.0
        self.corU.all_values[0, :] = 0.0
        self.corV.all_values[:, 0] = 0.0
        self.corV.all_values[-1, :] = 0.0
        if three_d:
            self.corpk.all_values[:, :, -1] = 0.0
            self.corpk.all_values[:, 0, :] = 0.0
            self.corqk.all_values[:, :, 0] = 0.0
            self.corqk.all_values[:, -1, :] = 0.0
        if self.advection_scheme is None:
            self.advection_scheme = default_advection_scheme
        inc2d = "float32" if self.dtype3d == torch.float32 else "float64"
        self.uadv = Advection(ug, scheme=self.advection_scheme, split_2d=self.advection_split_2d, increments_2d=inc2d)
        self.vadv = Advection(vg, scheme=self.advection_scheme, split_2d=self.advection_split_2d, increments_2d=inc2d)
        if three_d:
            self.hU_bot = ug.hn.isel(z=0)
            self.hV_bot = vg.hn.isel(z=0)
            if self.dtype3d == torch.float64:
                self.u_bot = self.uk.isel(z=0)
                self.v_bot = self.vk.isel(z=0)
            else:
                self.u_bot, self.v_bot = self._u_bot64, self._v_bot64
            self._vertical_diffusion = VerticalDiffusion(tgrid, cnpar=self.cnpar)
            self.ea2 = tgrid.array(fill=0.0, z=CENTERS, dtype=self.dtype3d)
            self.ea4 = tgrid.array(fill=0.0, z=CENTERS, dtype=self.dtype3d)
        self.An = tgrid.array(name="An")
        self.An.fill(self._An_const)
        self._ufirst = False
        self._u3dfirst = False
        self.An_uu = self.An_uv = self.An_vu = self.An_vv = None

    def start(self):
        """momentum.py:618-642"""
        zero = MASK_ZERO_2D + (MASK_ZERO_3D if self.runtype > 1 else ())
        for n in zero:
            a = getattr(self, n)
            a.all_values[..., a.grid.land] = 0.0
        self.An.all_values[self.An.grid.land] = FILL_VALUE
        if bool((self.An.all_values[self.An.grid.water] == 0.0).all()):
            self.An_uu = self.An_uv = self.An_vu = self.An_vv = None
        else:
            nan = float("nan")
            self.An_uu = self.An.interp(self.U.grid.ugrid.array(fill=nan))
            self.An_uv = self.An.interp(self.U.grid.vgrid.array(fill=nan))
            self.An_vu = self.An.interp(self.V.grid.ugrid.array(fill=nan))
            self.An_vv = self.An.interp(self.V.grid.vgrid.array(fill=nan))

    # ------------------------------------------------------------------ 2D
    def advance_depth_integrated(self, timestep: float, tausx: Array, tausy: Array, dpdx: Array, dpdy: Array):
        """momentum.py:644-718"""

        mixed = self.fused_2d and self.dtype3d == torch.float32

        def u():
            _pygetm.advance_2d_transport(self.U, dpdx, tausx, self.corU, self.advU, self.diffU, self.dampU,
                                         self.SxA, self.SxB, self.SxD, self.SxF, self.ru, timestep, mixed)
            if self._ob is not None:
                self._ob.mirror("U", self.U)
            self.coriolis(self.U, self.corV, True)

        def v():
            _pygetm.advance_2d_transport(self.V, dpdy, tausy, self.corV, self.advV, self.diffV, self.dampV,
                                         self.SyA, self.SyB, self.SyD, self.SyF, self.rv, timestep, mixed)
            if self._ob is not None:
                self._ob.mirror("V", self.V)
            self.coriolis(self.V, self.corU, False)

        if self._ufirst:
            u()
            v()
        else:
            v()
            u()
        self._ufirst = not self._ufirst
        if self.runtype > 1:
            if self.fused_2d:
                _pygetm.accumulate_2d(self.U, self.V, self._U_cum, self._V_cum)
            else:
                self._U_cum += self.U.all_values
                self._V_cum += self.V.all_values

    def update_depth_integrated_diagnostics(self, timestep: float, skip_coriolis: bool = False,
                                            update_z0b: bool = False):
        """momentum.py:720-758"""
        if not skip_coriolis:
            self.coriolis(self.U, self.corV, True)
            self.coriolis(self.V, self.corU, False)
        self._transport_2d_momentum(self.U, self.V, timestep, self.advU, self.advV, self.diffU, self.diffV, update_z0b)
        if self.An_uu is not None:
            _pygetm.horizontal_diffusion(self.U, self.An_uu, self.An_uv, timestep, self.dampU)
            _pygetm.horizontal_diffusion(self.V, self.An_vu, self.An_vv, timestep, self.dampV)

    def _transport_2d_momentum(self, U: Array, V: Array, timestep: float, advU: Array, advV: Array,
                               diffU: Array, diffV: Array, update_z0b: bool):
        """momentum.py:1017-1097"""
        if self.fused_2d and not update_z0b:
            self._transport_2d_momentum_fused(U, V, timestep, advU, advV, diffU, diffV)
            return
        torch.div(U.all_values, U.grid.D.all_values, out=self.u1.all_values)
        torch.div(V.all_values, V.grid.D.all_values, out=self.v1.all_values)
        if self.diffuse_momentum:
            _pygetm.momentum_diffusion(self.uua.grid.D, self.uva.grid.D, self.vua.grid.D, self.vva.grid.D,
                                       self.u1, self.v1, self._Am_const, diffU, diffV)
        if self.apply_bottom_friction:
            self.bottom_friction(self.u1, self.v1, self.u1.grid.D, self.v1.grid.D, self.ru, self.rv, update_z0b)
        U.interp(self.uua)
        V.interp(self.uva)
        self.uua.all_values.div_(self.uua.grid.D.all_values)
        self.uva.all_values.div_(self.uva.grid.D.all_values)
        advU.all_values.copy_(self.u1.all_values)
        self.uadv(self.uua, self.uva, timestep, advU, skip_initial_halo_exchange=True)
        _pygetm.reconstruct_transport_change(advU, self.uadv.D, U, timestep)
        U.interp(self.vua)
        V.interp(self.vva)
        self.vua.all_values.div_(self.vua.grid.D.all_values)
        self.vva.all_values.div_(self.vva.grid.D.all_values)
        advV.all_values.copy_(self.v1.all_values)
        self.vadv(self.vua, self.vva, timestep, advV, skip_initial_halo_exchange=True)
        _pygetm.reconstruct_transport_change(advV, self.vadv.D, V, timestep)

    def _transport_2d_momentum_fused(self, U, V, timestep, advU, advV, diffU, diffV):
        """The same sequence with two fused kernels for everything before the
        advection calls (velocities and copies; drag coefficients)."""
        mixed = self.dtype3d == torch.float32
        _pygetm.momentum_2d_velocities(U, V, self.u1, self.v1, advU, advV, self.uua, self.uva, self.vua, self.vva,
                                       mixed)
        if self.diffuse_momentum:
            _pygetm.momentum_diffusion(self.uua.grid.D, self.uva.grid.D, self.vua.grid.D, self.vva.grid.D,
                                       self.u1, self.v1, self._Am_const, diffU, diffV)
        if self.apply_bottom_friction:
            _pygetm.momentum_2d_friction(self.u1, self.v1, self.ru, self.rv, mixed)
        self.uadv(self.uua, self.uva, timestep, advU, skip_initial_halo_exchange=True)
        _pygetm.reconstruct_transport_change(advU, self.uadv.D, U, timestep)
        self.vadv(self.vua, self.vva, timestep, advV, skip_initial_halo_exchange=True)
        _pygetm.reconstruct_transport_change(advV, self.vadv.D, V, timestep)

    def bottom_friction(self, u: Array, v: Array, DU: Array, DV: Array, ru: Array, rv: Array,
                        update_z0b: bool = False):
        """momentum.py:1099-1125"""
        u_V = u.interp(v.grid._work)
        v_U = v.interp(u.grid._work)
        ar = "float32" if self.dtype3d == torch.float32 else "float64"
        _pygetm.bottom_friction(u, v_U, DU, self.avmmol, ru, update_z0b, ar)
        _pygetm.bottom_friction(u_V, v, DV, self.avmmol, rv, update_z0b, ar)

    def coriolis(self, U: Array, out: Array, x_direction: bool):
        """momentum.py:1127-1148 (DEFAULT and ESPELID schemes)"""
        assert U.grid is not out.grid
        if self.coriolis_scheme == CoriolisScheme.ESPELID:
            _pygetm.coriolis_espelid(U, out, x_direction)
            return
        if self.fused_2d and not U.z:
            _pygetm.coriolis_2d(U, out, x_direction, mixed=self.dtype3d == torch.float32)
            return
        if self.fused_2d:
            _pygetm.coriolis_3d(U, out, x_direction)
            return
        U.interp(out)
        out.all_values.mul_(out.grid.cor.all_values)
        if x_direction:
            out.all_values.neg_()

    # ------------------------------------------------------------------ 3D
    def advance(self, timestep: float, split_factor: int, tausx: Array, tausy: Array, dpdx: Array, dpdy: Array,
                idpdx: Array, idpdy: Array, viscosity: Array, side_stream=None):
        """momentum.py:760-858.  ``side_stream``: see update_diagnostics."""
        _pygetm.mean_transports(self._U_cum, self._V_cum, 1.0 / split_factor, self.Ui, self.Vi)

        def u():
            self.advance_3d_transport(self.pk, self.Ui, self.uk, dpdx, self.corpk, self.advpk, self.diffpk, idpdx,
                                      tausx, self.rru, viscosity, self.udev, timestep, self._visc_u)
            self.coriolis(self.pk, self.corqk, True)

        def v():
            self.advance_3d_transport(self.qk, self.Vi, self.vk, dpdy, self.corqk, self.advqk, self.diffqk, idpdy,
                                      tausy, self.rrv, viscosity, self.vdev, timestep, self._visc_v)
            self.coriolis(self.qk, self.corpk, False)

        if self._u3dfirst:
            u()
            v()
        else:
            v()
            u()
        self._u3dfirst = not self._u3dfirst
        self.update_diagnostics(timestep, viscosity, skip_coriolis=True, side_stream=side_stream)

    def update_diagnostics(self, timestep: float, viscosity: Array, skip_coriolis: bool = False,
                           side_stream=None):
        """momentum.py:860-1015.  ``side_stream``: a CUDA stream on which
        everything after the 3D velocities and the vertical velocity is
        issued (shear frequency SS, bottom drag rru/rrv and shear velocities,
        the advection of the 3D momentum and the slow terms advpk, advqk,
        SxA, SyA, SxD, SyD, SxF, SyF); the caller joins it
        (current_stream().wait_stream) before anything reads those or the
        momentum advection handles and 2D work arrays they use."""
        if not skip_coriolis:
            self.coriolis(self.pk, self.corqk, True)
            self.coriolis(self.qk, self.corpk, False)
        _pygetm.w_momentum_3d(self.pk, self.qk, timestep, self.ww)
        if self.u_bot is self._u_bot64:  # mixed form: the FP64 bottom velocities in the same launch
            _pygetm.velocities_3d(self.pk, self.qk, self.uk, self.vk, self._u_bot64, self._v_bot64)
        else:
            _pygetm.velocities_3d(self.pk, self.qk, self.uk, self.vk)
        if side_stream is None:
            self._diagnostics_tail(timestep)
            return
        side_stream.wait_stream(torch.cuda.current_stream(side_stream.device))
        with torch.cuda.stream(side_stream):
            self._diagnostics_tail(timestep, self._v_stream)

    def _diagnostics_tail(self, timestep: float, v_stream=None):
        """update_diagnostics after the velocities (momentum.py:880-1015):
        shear frequency, bottom stress, advection of the 3D momentum, its
        depth-integrated counterpart and the slow terms.  ``v_stream``: a
        stream on which the advection of the V momentum runs beside that of
        the U momentum (separate handles, inputs and outputs)."""
        _pygetm.shear_frequency(self.uk, self.vk, self.SS)
        if self.apply_bottom_friction:
            self.bottom_friction(self.u_bot, self.v_bot, self.hU_bot, self.hV_bot, self.rru, self.rrv)
        _pygetm.bottom_shear_velocity(self.u_bot, self.v_bot, self.rru, self.rrv, self.ustar2_bx, self.ustar2_by,
                                      self.ustar_b)
        # SS and ustar_b are ready: a turbulence closure on another stream
        # may start from here
        self._bottom_event.record()
        # advpk = uk, advqk = vk and the velocities on the advection grids
        # (the interpolations below, all at once)
        _pygetm.momentum_3d_advection_inputs(self.uk, self.vk, self.ww, self.uua3d, self.uva3d, self.vua3d,
                                             self.vva3d, self._ww_u, self._ww_v, self.advpk, self.advqk)
        def v_advection():
            self.vadv.apply_3d(self.vua3d, self.vva3d, self._ww_v,
                               timestep, self.advqk, new_h=True, skip_initial_halo_exchange=True)
            _pygetm.reconstruct_transport_change(self.advqk, self.vadv.h, self.qk, timestep)

        here = torch.cuda.current_stream(self.uk.all_values.device) if v_stream is not None else None
        if v_stream is not None:
            v_stream.wait_stream(here)
            with torch.cuda.stream(v_stream):
                v_advection()
        self.uadv.apply_3d(self.uua3d, self.uva3d, self._ww_u,
                           timestep, self.advpk, new_h=True, skip_initial_halo_exchange=True)
        _pygetm.reconstruct_transport_change(self.advpk, self.uadv.h, self.pk, timestep)
        if v_stream is None:
            v_advection()
        else:
            here.wait_stream(v_stream)
        if self.diffuse_momentum:
            _pygetm.momentum_diffusion(self.uua.grid.hn, self.uva.grid.hn, self.vua.grid.hn, self.vva.grid.hn,
                                       self.uk, self.vk, self._Am_const, self.diffpk, self.diffqk)
        self._transport_2d_momentum(self.Ui, self.Vi, timestep, self.SxA, self.SyA, self.SxD, self.SyD, False)
        # SxA = sum_k advpk - SxA, ... (the column sums in FP64)
        _pygetm.column_sums([(self.advpk, self.SxA), (self.advqk, self.SyA), (self.diffpk, self.SxD),
                             (self.diffqk, self.SyD)], subtract=True)
        if self.apply_bottom_friction:
            _pygetm.slow_friction(self.ustar2_bx, self.ru, self.u1, self.SxF, self.ustar2_by, self.rv, self.v1,
                                  self.SyF)

    def advance_3d_transport(self, tp3d: Array, tp2d: Array, vel3d: Array, dp: Array, cor: Array, adv: Array,
                             diff: Array, idp: Array, taus: Array, rr: Array, viscosity: Array, dev: Array,
                             timestep: float, visc_target: Optional[Array] = None):
        """momentum.py:1164-1214"""
        grid = tp3d.grid
        _pygetm.collect_3d_momentum_sources(dp, cor, adv, diff, idp, taus, rr, timestep, self.ea2, self.ea4)
        visc = viscosity.interp(visc_target if visc_target is not None else grid)
        self._vertical_diffusion(visc, timestep, vel3d, molecular=self.avmmol, ea2=self.ea2, ea4=self.ea4,
                                 use_ho=True)
        # tp3d = vel3d hn; dev = (sum_k tp3d - tp2d) / D; tp3d -= dev hn
        _pygetm.transport_3d_finish(vel3d, grid.hn, tp2d, grid.D, tp3d, dev)
        if self._ob is not None:  # momentum.py:1211-1212
            self._ob.mirror("U" if tp3d is self.pk else "V", tp3d)
