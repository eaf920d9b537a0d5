"""Oracle time-step drivers (numpy + C restatement) - TEST INFRASTRUCTURE ONLY.

``TracerTransport`` restates TracerCollection.advance / _diffuse
(python/pygetm/tracer.py:193-276) on the oracle operators, started from the
same ``Workload`` arrays as the GPU driver.
"""

from __future__ import annotations

import numpy as np

from . import oracle as O
from . import turbulence


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


# ---------------------------------------------------------------------------
# Split-explicit baroclinic step: restatement of python/pygetm/simulation.py
# (Simulation.__init__/_start/_advance_state/_update_forcing_and_diagnostics/
# update_depth) and python/pygetm/momentum.py (Momentum) for closed domains,
# constant surface fluxes, prescribed vertical mixing and Sigma coordinates.
# ---------------------------------------------------------------------------
FILL = O.FILL_VALUE
NAN = float("nan")


def _arr(g, nz=None, fill=None):
    """Array.create (python/pygetm/core.py:853-900): explicit fill everywhere,
    else FILL_VALUE; nz None = 2D, else number of levels."""
    shape = (g.ny_, g.nx_) if nz is None else (nz, g.ny_, g.nx_)
    return np.full(shape, FILL if fill is None else fill)


def _fill(a, g, value, fill_value=FILL):
    """Array.fill (python/pygetm/core.py:901-911)."""
    a[...] = value
    a[..., g.land] = fill_value


def totals(T, D, hn, tracers):
    """Simulation.totals (python/pygetm/simulation.py:1409-1444) with
    Array.global_sum on one subdomain (python/pygetm/core.py:820-839):
    [sum of D * area, then per tracer sum of c * area * hn], each over the
    interior points where mask != 0 (numpy's pairwise sum, as the reference)."""
    i = T.interior
    unmasked = T.mask[i] != 0
    out = [float((D * T.area)[i].sum(where=unmasked))]
    for c in tracers:
        tot = np.asarray(c, dtype=float) * T.area * hn
        out.append(float(tot[i].sum(where=np.broadcast_to(unmasked, tot[i].shape))))
    return out


def seos_buoyancy(S, T, z):
    """Device EOS restated (simplified nonlinear EOS of Roquet et al. 2015);
    buoyancy -g/rho0 (rho - rho0) as python/pygetm/simulation.py:1184."""
    Ta = T - 10.0
    Sa = S - 35.0
    rho = (1026.0 - 1.6550e-1 * (1.0 + 0.5 * 5.9520e-2 * Ta + 1.4970e-4 * z) * Ta
           + 7.6554e-1 * (1.0 - 0.5 * 5.4914e-4 * Sa - 1.1090e-5 * z) * Sa - 2.4341e-3 * Ta * Sa)
    return rho, (-O.GRAVITY / O.RHO0) * (rho - O.RHO0)


def seos_nsquared(mask, h, p, S, T):
    """Squared buoyancy frequency of the device EOS at the interior interfaces
    (Density.get_buoyancy_frequency, python/pygetm/density.py:22-60):
    -g/rho0 (rho(S1, T1, zi) - rho(S0, T0, zi)) / dz, both densities at the
    mean depth zi of the two layer centres, dz the mean thickness.  Returns
    the (nz - 1) interior interfaces; NaN where the mask is zero."""
    S0, S1, T0, T1 = S[:-1], S[1:], T[:-1], T[1:]
    zi = 0.5 * (p[:-1] + p[1:])
    dz = 0.5 * (h[:-1] + h[1:])
    rho1, _ = seos_buoyancy(S1, T1, zi)
    rho0, _ = seos_buoyancy(S0, T0, zi)
    out = (-O.GRAVITY / O.RHO0) * (rho1 - rho0) / dz
    return np.where(np.asarray(mask)[None] != 0, out, np.nan)


class Momentum:
    """python/pygetm/momentum.py:24-1214 (DEFAULT Coriolis, FULL 2D split)."""

    def __init__(self, Am=0.0, An=0.0, cnpar=1.0, advection_scheme=None, avmmol=1.8e-6, coriolis_scheme=1):
        """coriolis_scheme: 1 DEFAULT, 2 ESPELID (momentum.py:14-17)."""
        self._Am_const, self._An_const, self.cnpar = Am, An, cnpar
        self.advection_scheme = advection_scheme
        self.avmmol = avmmol
        self.coriolis_scheme = coriolis_scheme

    def initialize(self, T, runtype, default_scheme):
        ug, vg = T.ugrid, T.vgrid
        self.runtype = runtype
        for n in ("U", "u1", "SxA", "SxB", "SxD", "SxF", "corU", "advU", "diffU", "dampU", "ru"):
            setattr(self, n, _arr(ug))
        for n in ("V", "v1", "SyA", "SyB", "SyD", "SyF", "corV", "advV", "diffV", "dampV", "rv"):
            setattr(self, n, _arr(vg))
        self.uua, self.uva = _arr(ug.ugrid, fill=NAN), _arr(ug.vgrid, fill=NAN)
        self.vua, self.vva = _arr(vg.ugrid, fill=NAN), _arr(vg.vgrid, fill=NAN)
        nz = T.nz
        for n in ("pk", "uk", "corpk", "advpk", "diffpk"):
            setattr(self, n, _arr(ug, nz))
        for n in ("qk", "vk", "corqk", "advqk", "diffqk"):
            setattr(self, n, _arr(vg, nz))
        self.ww = _arr(T, nz + 1)
        self.SS = _arr(T, nz + 1)
        for n in ("rru", "Ui", "udev", "ustar2_bx"):
            setattr(self, n, _arr(ug))
        for n in ("rrv", "Vi", "vdev", "ustar2_by"):
            setattr(self, n, _arr(vg))
        self._U_cum = np.zeros_like(self.Ui)
        self._V_cum = np.zeros_like(self.Vi)
        self.uua3d, self.uva3d = _arr(ug.ugrid, nz, NAN), _arr(ug.vgrid, nz, NAN)
        self.vua3d, self.vva3d = _arr(vg.ugrid, nz, NAN), _arr(vg.vgrid, nz, NAN)
        self.ustar_b = _arr(T)
        self.apply_bottom_friction = not ((ug.z0b_min[ug.water] == 0.0).any() or (vg.z0b_min[vg.water] == 0.0).any())
        self.diffuse_momentum = self._Am_const > 0.0
        grids = dict(U=ug, u1=ug, V=vg, v1=vg, pk=ug, qk=vg, uk=ug, vk=vg, Ui=ug, Vi=vg, rru=ug, rrv=vg)
        for n in ("U", "V", "u1", "v1", "pk", "qk", "uk", "vk", "Ui", "Vi", "rru", "rrv"):
            getattr(self, n)[...] = 0.0
        for n, g in (("SxA", ug), ("SyA", vg), ("SxB", ug), ("SyB", vg), ("SxD", ug), ("SyD", vg), ("SxF", ug),
                     ("SyF", vg), ("dampU", ug), ("dampV", vg), ("advU", ug), ("advV", vg), ("diffU", ug),
                     ("diffV", vg), ("ru", ug), ("rv", vg), ("corU", ug), ("corV", vg), ("SS", T), ("advpk", ug),
                     ("advqk", vg), ("diffpk", ug), ("diffqk", vg), ("corpk", ug), ("corqk", vg), ("ww", T)):
            _fill(getattr(self, n), g, 0.0)
        self.corU[:, -1] = 0.0
        self.corU[0, :] = 0.0
        self.corV[:, 0] = 0.0
        self.corV[-1, :] = 0.0
        self.corpk[:, :, -1] = 0.0
        self.corpk[:, 0, :] = 0.0
        self.corqk[:, :, 0] = 0.0
        self.corqk[:, -1, :] = 0.0
        scheme = self.advection_scheme or default_scheme
        self.uadv = O.Advection(ug, scheme, O.AdvectionSplit.FULL)
        self.vadv = O.Advection(vg, scheme, O.AdvectionSplit.FULL)
        self.vdif = O.VerticalDiffusion(T, cnpar=self.cnpar)
        self.ea2 = np.zeros((nz, T.ny_, T.nx_))
        self.ea4 = np.zeros((nz, T.ny_, T.nx_))
        self._grids = grids
        self._ufirst = False
        self._u3dfirst = False
        self.ob = None  # open-boundary operations (set by the simulation)
        self._T = T
        self.An = _arr(T)
        _fill(self.An, T, self._An_const)
        self.An_uu = self.An_uv = self.An_vu = self.An_vv = None

    def start(self):
        for n, g in self._grids.items():
            a = getattr(self, n)
            a[..., g.land] = 0.0
        # momentum.py:630-642: numerical damping only where An is non-zero
        T = self._T
        self.An[T.land] = FILL
        if (self.An[T.water] == 0.0).all():
            self.An_uu = self.An_uv = self.An_vu = self.An_vv = None
        else:
            ug, vg = T.ugrid, T.vgrid
            self.An_uu, self.An_uv = _arr(ug.ugrid, fill=NAN), _arr(ug.vgrid, fill=NAN)
            self.An_vu, self.An_vv = _arr(vg.ugrid, fill=NAN), _arr(vg.vgrid, fill=NAN)
            for tgt, g in ((self.An_uu, ug.ugrid), (self.An_uv, ug.vgrid), (self.An_vu, vg.ugrid),
                           (self.An_vv, vg.vgrid)):
                O.interpolate(T, g, self.An, tgt)

    def coriolis(self, src_grid, U, out_grid, out, x_direction):
        """momentum.py:1127-1148.  ESPELID: interp(U / sqrt(Din)) * sqrt(Dout),
        D the water depth (2D) or layer thickness (3D); sqrt(Din) is 1 on
        land.  The reference leaves the sqrt(Dout) factor unset on land
        points of the target (np.sqrt with where= and no out=); it is left
        out there, and nothing reads those points."""
        if self.coriolis_scheme == 2:
            Din = src_grid.D if U.ndim == 2 else src_grid.hn
            Dout = out_grid.D if out.ndim == 2 else out_grid.hn
            with np.errstate(invalid="ignore"):
                sqrtDin = np.where(src_grid.mask != 0, np.sqrt(Din), 1.0)
            O.interpolate(src_grid, out_grid, U / sqrtDin, out)
            wet = np.broadcast_to(out_grid.mask != 0, out.shape)
            out[wet] *= np.sqrt(Dout[wet])
        else:
            O.interpolate(src_grid, out_grid, U, out)
        out *= out_grid.cor
        if x_direction:
            np.negative(out, out=out)

    def advance_depth_integrated(self, T, timestep, tausx, tausy, dpdx, dpdy):
        ug, vg = T.ugrid, T.vgrid

        def u():
            O.advance_2d_transport(ug, self.U, dpdx, tausx, self.corU, self.advU, self.diffU, self.dampU, self.SxA,
                                   self.SxB, self.SxD, self.SxF, self.ru, timestep)
            if self.ob is not None:
                self.ob.mirror("U", self.U)
            self.coriolis(ug, self.U, vg, self.corV, True)

        def v():
            O.advance_2d_transport(vg, self.V, dpdy, tausy, self.corV, self.advV, self.diffV, self.dampV, self.SyA,
                                   self.SyB, self.SyD, self.SyF, self.rv, timestep)
            if self.ob is not None:
                self.ob.mirror("V", self.V)
            self.coriolis(vg, self.V, ug, self.corU, False)

        if self._ufirst:
            u(); v()
        else:
            v(); u()
        self._ufirst = not self._ufirst
        self._U_cum += self.U
        self._V_cum += self.V

    def update_depth_integrated_diagnostics(self, T, timestep, skip_coriolis=False):
        if not skip_coriolis:
            self.coriolis(T.ugrid, self.U, T.vgrid, self.corV, True)
            self.coriolis(T.vgrid, self.V, T.ugrid, self.corU, False)
        self._transport_2d_momentum(T, self.U, self.V, timestep, self.advU, self.advV, self.diffU, self.diffV)
        if self.An_uu is not None:  # numerical damping (momentum.py:751-758)
            O.horizontal_diffusion(T.ugrid, self.U, self.An_uu, self.An_uv, timestep, self.dampU)
            O.horizontal_diffusion(T.vgrid, self.V, self.An_vu, self.An_vv, timestep, self.dampV)

    def _transport_2d_momentum(self, T, U, V, timestep, advU, advV, diffU, diffV):
        ug, vg = T.ugrid, T.vgrid
        with np.errstate(all="ignore"):
            np.divide(U, ug.D, out=self.u1)
            np.divide(V, vg.D, out=self.v1)
        if self._Am_const > 0.0:  # momentum.py:1051-1064
            O.momentum_diffusion(ug, vg, ug.ugrid.D, ug.vgrid.D, vg.ugrid.D, vg.vgrid.D, self.u1, self.v1,
                                 self._Am_const, diffU, diffV)
        if self.apply_bottom_friction:
            self.bottom_friction(T, self.u1, self.v1, ug.D, vg.D, self.ru, self.rv)
        with np.errstate(all="ignore"):
            O.interpolate(ug, ug.ugrid, U, self.uua)
            O.interpolate(vg, ug.vgrid, V, self.uva)
            self.uua /= ug.ugrid.D
            self.uva /= ug.vgrid.D
            advU[...] = self.u1
            self.uadv(self.uua, self.uva, timestep, advU)
            O.reconstruct_transport_change(ug, advU, self.uadv.D, U, timestep)
            O.interpolate(ug, vg.ugrid, U, self.vua)
            O.interpolate(vg, vg.vgrid, V, self.vva)
            self.vua /= vg.ugrid.D
            self.vva /= vg.vgrid.D
            advV[...] = self.v1
            self.vadv(self.vua, self.vva, timestep, advV)
            O.reconstruct_transport_change(vg, advV, self.vadv.D, V, timestep)

    def bottom_friction(self, T, u, v, DU, DV, ru, rv):
        ug, vg = T.ugrid, T.vgrid
        u_V = np.full((vg.ny_, vg.nx_), NAN)
        v_U = np.full((ug.ny_, ug.nx_), NAN)
        O.interpolate(ug, vg, u, u_V)
        O.interpolate(vg, ug, v, v_U)
        O.bottom_friction(ug, np.ascontiguousarray(u), v_U, np.ascontiguousarray(DU), self.avmmol, ru, False)
        O.bottom_friction(vg, u_V, np.ascontiguousarray(v), np.ascontiguousarray(DV), self.avmmol, rv, False)

    def advance(self, T, timestep, split_factor, tausx, tausy, dpdx, dpdy, idpdx, idpdy, viscosity):
        ug, vg = T.ugrid, T.vgrid
        np.multiply(self._U_cum, 1.0 / split_factor, out=self.Ui)
        np.multiply(self._V_cum, 1.0 / split_factor, out=self.Vi)
        self._U_cum.fill(0.0)
        self._V_cum.fill(0.0)

        def u():
            self.advance_3d_transport(T, ug, self.pk, self.Ui, self.uk, dpdx, self.corpk, self.advpk, self.diffpk,
                                      idpdx, tausx, self.rru, viscosity, self.udev, timestep)
            self.coriolis(ug, self.pk, vg, self.corqk, True)

        def v():
            self.advance_3d_transport(T, vg, self.qk, self.Vi, self.vk, dpdy, self.corqk, self.advqk, self.diffqk,
                                      idpdy, tausy, self.rrv, viscosity, self.vdev, timestep)
            self.coriolis(vg, self.qk, ug, self.corpk, False)

        if self._u3dfirst:
            u(); v()
        else:
            v(); u()
        self._u3dfirst = not self._u3dfirst
        self.update_diagnostics(T, timestep, viscosity, skip_coriolis=True)

    def update_diagnostics(self, T, timestep, viscosity, skip_coriolis=False):
        ug, vg = T.ugrid, T.vgrid
        if not skip_coriolis:
            self.coriolis(ug, self.pk, vg, self.corqk, True)
            self.coriolis(vg, self.qk, ug, self.corpk, False)
        O.w_momentum_3d(T, self.pk, self.qk, timestep, self.ww)
        with np.errstate(all="ignore"):
            np.divide(self.pk, ug.hn, out=self.uk)
            np.divide(self.qk, vg.hn, out=self.vk)
        O.shear_frequency(T, self.uk, self.vk, self.SS)
        u_bot = np.ascontiguousarray(self.uk[0])
        v_bot = np.ascontiguousarray(self.vk[0])
        if self.apply_bottom_friction:
            self.bottom_friction(T, u_bot, v_bot, ug.hn[0], vg.hn[0], self.rru, self.rrv)
        O.bottom_shear_velocity(T, u_bot, v_bot, self.rru, self.rrv, self.ustar2_bx, self.ustar2_by, self.ustar_b)
        nz = T.nz
        with np.errstate(all="ignore"):
            self.advpk[...] = self.uk
            O.interpolate(ug, ug.ugrid, self.uk, self.uua3d)
            O.interpolate(vg, ug.vgrid, self.vk, self.uva3d)
            ww_u = np.zeros((nz + 1, ug.ny_, ug.nx_))
            O.interpolate(T, ug, self.ww, ww_u)
            self.uadv.apply_3d(self.uua3d, self.uva3d, ww_u, timestep, self.advpk, new_h=True)
            O.reconstruct_transport_change(ug, self.advpk, self.uadv.h, self.pk, timestep)
            self.advqk[...] = self.vk
            O.interpolate(ug, vg.ugrid, self.uk, self.vua3d)
            O.interpolate(vg, vg.vgrid, self.vk, self.vva3d)
            ww_v = np.zeros((nz + 1, vg.ny_, vg.nx_))
            O.interpolate(T, vg, self.ww, ww_v)
            self.vadv.apply_3d(self.vua3d, self.vva3d, ww_v, timestep, self.advqk, new_h=True)
            O.reconstruct_transport_change(vg, self.advqk, self.vadv.h, self.qk, timestep)
        if self._Am_const > 0.0:  # momentum.py:963-978
            O.momentum_diffusion(ug, vg, ug.ugrid.hn, ug.vgrid.hn, vg.ugrid.hn, vg.vgrid.hn, self.uk, self.vk,
                                 self._Am_const, self.diffpk, self.diffqk)
        self._transport_2d_momentum(T, self.Ui, self.Vi, timestep, self.SxA, self.SyA, self.SxD, self.SyD)
        self.SxA[...] = self.advpk.sum(axis=0) - self.SxA
        self.SyA[...] = self.advqk.sum(axis=0) - self.SyA
        self.SxD[...] = self.diffpk.sum(axis=0) - self.SxD
        self.SyD[...] = self.diffqk.sum(axis=0) - self.SyD
        if self.apply_bottom_friction:
            self.SxF[...] = self.ustar2_bx + self.ru * self.u1
            self.SyF[...] = self.ustar2_by + self.rv * self.v1

    def advance_3d_transport(self, T, grid, tp3d, tp2d, vel3d, dp, cor, adv, diff, idp, taus, rr, viscosity, dev,
                             timestep):
        O.collect_3d_momentum_sources(grid, dp, cor, adv, diff, idp, taus, rr, timestep, self.ea2, self.ea4)
        visc = np.zeros((T.nz + 1, grid.ny_, grid.nx_))
        O.interpolate(T, grid, viscosity, visc)
        vd = O.VerticalDiffusion(grid, cnpar=self.cnpar)
        vd(visc, timestep, vel3d, molecular=self.avmmol, ea2=self.ea2, ea4=self.ea4, use_ho=True)
        with np.errstate(all="ignore"):
            np.multiply(vel3d, grid.hn, out=tp3d)
            tp3d.sum(axis=0, out=dev)
            dev -= tp2d
            dev /= grid.D
            tp3d -= dev * grid.hn
        if self.ob is not None:
            self.ob.mirror("U" if tp3d is self.pk else "V", tp3d)


class BoundaryOps:
    """Open-boundary conditions and mirroring restated in numpy
    (python/pygetm/open_boundaries.py: ZeroGradient :338-356, Clamped
    :358-375, Flather :377-416, Sponge :195-336 without flow-dependent
    relaxation; core.Array.mirror, core.py:723-728).  Boundaries are updated
    one after another, as ArrayOpenBoundaries.update does (:494-497)."""

    def __init__(self, ob, T):
        self.ob = ob
        self.T = T
        self.ranges = [(b.start, b.stop) for b in ob]
        self.z = np.zeros(ob.np)
        self.flow = np.zeros(ob.np)
        self.tracer_values = {}

    def prescribe(self, time):
        if self.ob.constituents:
            self.z[...] = 0.0
            for om, amp, ph in self.ob.constituents:
                self.z += amp * np.cos(time * om + ph)

    def update_elevation(self, sim):
        ob, T = self.ob, self.T
        z = T.z
        for s, e in self.ranges:
            i, j = ob.i[s:e], ob.j[s:e]
            ty = ob.type_2d[s]
            if ty == 1:  # ZERO_GRADIENT
                v = z[j + ob.dj[s:e], i + ob.di[s:e]]
            elif ty == 3:  # CLAMPED
                v = self.z[s:e]
            else:
                side = ob.side[s]
                U, V = sim.momentum.U, sim.momentum.V
                tp = {1: U[j, i], 3: U[j, i - 1], 4: V[j, i], 2: V[j - 1, i]}[side]
                D = T.Dclip[j, i]
                ext = self.flow[s:e] * D if ty == 4 else self.flow[s:e]
                v = self.z[s:e] - ob.inflow_sign[s:e] * (tp - ext) / np.sqrt(D * O.GRAVITY)
            z[j, i] = np.maximum(sim.Dmin - T.H[j, i], v)

    def mirror(self, name, field):
        src, tgt = getattr(self.ob, "mirror_" + name)
        if src.size:
            flat = field.reshape(field.shape[:-2] + (-1,))
            flat[..., tgt] = flat[..., src]

    def mirror_to(self, name, source, target):
        src, tgt = getattr(self.ob, "mirror_" + name)
        if src.size:
            target.reshape(target.shape[:-2] + (-1,))[..., tgt] = source.reshape(source.shape[:-2] + (-1,))[..., src]

    def init_tracer_values(self, tracers):
        ob = self.ob
        for n, tr in enumerate(tracers):
            self.tracer_values[n] = tr[:, ob.j, ob.i].copy()

    def update_zero_gradient(self, field):
        """ArrayOpenBoundaries.update of an array whose boundaries are all
        ZERO_GRADIENT (num, python/pygetm/vertical_mixing.py:120,186)."""
        ob = self.ob
        for s, e in self.ranges:
            i, j, di, dj = ob.i[s:e], ob.j[s:e], ob.di[s:e], ob.dj[s:e]
            field[:, j, i] = field[:, j + dj, i + di]

    def update_tracers(self, tracers):
        ob, T = self.ob, self.T
        n_sp = ob.sponge_n
        for n, tr in enumerate(tracers):
            bdyv = self.tracer_values[n]
            for s, e in self.ranges:
                i, j, di, dj = ob.i[s:e], ob.j[s:e], ob.di[s:e], ob.dj[s:e]
                ty = ob.type_3d[s]
                if ty == 1:
                    tr[:, j, i] = tr[:, j + dj, i + di]
                    continue
                b = bdyv[:, s:e]
                tr[:, j, i] = b
                if ty == 5:
                    for m in range(n_sp):
                        jj, ii = j + (m + 1) * dj, i + (m + 1) * di
                        sp = ((n_sp - m) / (n_sp + 1.0)) ** 2 * (T.mask[jj, ii] == 1)
                        tr[:, jj, ii] += sp * (b - tr[:, jj, ii])


class Simulation:
    """Restatement of pygetm.Simulation for the baroclinic split-explicit step
    (BAROCLINIC or BAROTROPIC_3D), matching getm_gb300.simulation.Simulation."""

    def __init__(self, T_host, dga, runtype=4, scheme=5, Dmin=0.02, Dcrit=0.1, num=0.0, nuh=0.0, taux=0.0, tauy=0.0,
                 sp=101325.0, internal_pressure="shchepetkin_mcwilliams", momentum=None, keps=None):
        """keps: None (prescribed num and nuh) or a dict of k-epsilon
        parameters (empty for the defaults): num and nuh from the closure of
        turbulence.keps_advance, advanced after the 3D momentum
        (python/pygetm/simulation.py:1107-1115)."""
        self.runtype = runtype
        self.dga = np.asarray(dga, dtype=float)[:, None, None]
        self.T = T = O.make_grids(T_host)
        self.U, self.V, self.X = T.ugrid, T.vgrid, T.xgrid
        self.Dmin, self.Dcrit = Dmin, Dcrit
        T.z = _arr(T); T.zo = _arr(T)
        _fill(T.z, T, 0.0); _fill(T.zo, T, 0.0)
        T.zin = _arr(T); T.zio = _arr(T)
        for g in (T, self.U, self.V):
            g.ho = _arr(g, T.nz)
        T.Dclip = _arr(T)
        T._work = _arr(T, fill=NAN)
        for g in (self.U, self.V, self.X):
            g._work = _arr(g, fill=NAN)
        self.h_T_half = _arr(T, T.nz, NAN)
        self.depth = _arr(T, T.nz)
        self.momentum = momentum or Momentum()
        self.momentum.initialize(T, runtype, scheme)
        self.taux = _arr(T); _fill(self.taux, T, taux)
        self.tauy = _arr(T); _fill(self.tauy, T, tauy)
        self.sp = _arr(T); _fill(self.sp, T, sp)
        self.pe = _arr(T); _fill(self.pe, T, 0.0)
        self.dpdx, self.dpdy = _arr(self.U), _arr(self.V)
        self.tausx, self.tausy = _arr(self.U), _arr(self.V)
        self.fwf = _arr(T); _fill(self.fwf, T, 0.0)
        self.num = _arr(T, T.nz + 1); _fill(self.num, T, num)
        self.nuh = _arr(T, T.nz + 1); _fill(self.nuh, T, nuh)
        self.ustar_s = _arr(T, fill=0.0)
        self.keps = None if keps is None else dict(keps)
        if self.keps is not None:
            # GOTM-style start: k = k_min, eps = eps_min everywhere
            self.tke, self.eps, self.L, nu_m, nu_h = turbulence.initial_state(T.nz, T.mask.shape, self.keps)
            for a in (self.tke, self.eps, self.L):  # Array.fill: land gets the fill value
                a[..., T.land] = FILL
            _fill(self.num, T, nu_m)
            _fill(self.nuh, T, nu_h)
            self.z0s = _arr(T, fill=0.1)
            self.NN = _arr(T, T.nz + 1, 0.0)
        self.tausxo, self.tausyo = np.zeros_like(self.tausx), np.zeros_like(self.tausy)
        self.dpdxo, self.dpdyo = np.zeros_like(self.dpdx), np.zeros_like(self.dpdy)
        self.adv = O.Advection(T, scheme)
        self.vdif = O.VerticalDiffusion(T, cnpar=1.0)
        self.tracers = []
        self.molecular = []
        if runtype == 4:
            self.temp = _arr(T, T.nz); _fill(self.temp, T, 5.0)
            self.salt = _arr(T, T.nz); _fill(self.salt, T, 35.0)
            self.tracers = [self.temp, self.salt]
            self.molecular = [1.4e-7, 1.1e-9]
            self.rho = _arr(T, T.nz)
            self.buoy = _arr(T, T.nz)
        self.internal_pressure_method = internal_pressure
        self.idpdx = _arr(self.U, T.nz); _fill(self.idpdx, self.U, 0.0)
        self.idpdy = _arr(self.V, T.nz); _fill(self.idpdy, self.V, 0.0)
        ob = getattr(T_host, "open_boundaries", None)
        self.ob = BoundaryOps(ob, T) if ob is not None and ob.np > 0 else None
        self.momentum.ob = self.ob
        self.time = 0.0
        self.update_depth(True)
        self.update_depth(True)

    def start(self, timestep, split_factor):
        self.timestep, self.split_factor = timestep, split_factor
        self.macrotimestep = timestep * split_factor
        self.istep = 0
        self.time = 0.0
        if self.ob is not None:
            self.ob.init_tracer_values(self.tracers)
        self._start()
        self._update_forcing_and_diagnostics(True)

    def advance(self):
        self.istep += 1
        self.time += self.timestep
        macro_active = self.istep % self.split_factor == 0
        self._advance_state(macro_active)
        self._update_forcing_and_diagnostics(macro_active)

    def _start(self):
        T = self.T
        self.momentum.start()
        for grid in (self.U, self.V):
            edges = grid.water_contact & grid.land
            grid.D[edges] = FILL
            grid.hn[..., edges] = FILL
        minz = -T.H + self.Dmin
        for z in (T.z, T.zo, T.zin, T.zio):
            shallow = (z < minz) & T.water
            np.putmask(z, shallow, minz)
        z_backup = T.z.copy()
        T.z[...] = T.zo
        self.update_depth(False)
        zin_backup = T.zin.copy()
        T.z[...] = T.zio
        _fill(T.zio, T, NAN)
        _fill(T.ho, T, NAN)
        self.update_depth(True)
        T.z[...] = zin_backup
        self.update_depth(True)
        self.momentum.update_diagnostics(T, self.macrotimestep, self.num)
        T.z[...] = z_backup

    def _advance_state(self, macro_active):
        T = self.T
        m = self.momentum
        m.advance_depth_integrated(T, self.timestep, self.tausx, self.tausy, self.dpdx, self.dpdy)
        T.zo[...] = T.z
        O.advance_surface_elevation(T, self.timestep, T.z, m.U, m.V, self.fwf)
        if macro_active:
            self.update_depth(True)
            m.advance(T, self.macrotimestep, self.split_factor, self.tausxo, self.tausyo, self.dpdxo, self.dpdyo,
                      self.idpdx, self.idpdy, self.num)
            if self.keps is not None:
                turbulence.keps_advance(T, self.macrotimestep, T.hn, self.ustar_s, m.ustar_b, self.z0s, T.z0b,
                                        self.NN, m.SS, self.tke, self.eps, self.L, self.num, self.nuh, self.keps)
                if self.ob is not None:
                    self.ob.update_zero_gradient(self.num)
            if self.tracers:
                self.adv.apply_3d_batch(m.uk, m.vk, m.ww, self.macrotimestep, self.tracers)
                avmol = -1.0
                for tr, mol in zip(self.tracers, self.molecular):
                    if mol != avmol:
                        avmol = mol
                        self.vdif.prepare(self.nuh, self.macrotimestep, avmol)
                    self.vdif.apply(tr)

    def _update_forcing_and_diagnostics(self, macro_active):
        T, m = self.T, self.momentum
        starting = self.istep == 0
        if macro_active and self.ob is not None:
            self.ob.update_tracers(self.tracers)
        if self.runtype == 4 and macro_active:
            with np.errstate(all="ignore"):
                self.rho[...], self.buoy[...] = seos_buoyancy(self.salt, self.temp, self.depth)
                if self.keps is not None:
                    N2 = seos_nsquared(T.mask, T.hn, self.depth, self.salt, self.temp)
                    self.NN[1:T.nz] = np.where(T.mask[None] != 0, N2, self.NN[1:T.nz])
            if self.internal_pressure_method == "blumberg_mellor":
                O.blumberg_mellor(T, self.buoy, self.idpdx, self.idpdy)
            else:
                O.shchepetkin_mcwilliams(T, self.buoy, self.idpdx, self.idpdy, T.zin)
            self.idpdx.sum(axis=0, out=m.SxB)
            self.idpdy.sum(axis=0, out=m.SyB)
        self.update_depth(False)
        m.update_depth_integrated_diagnostics(T, self.timestep, skip_coriolis=not starting)
        self.fwf[...] = self.pe
        if self.ob is not None:
            self.ob.prescribe(self.time)
            self.ob.update_elevation(self)
        O.surface_pressure_gradient(T, T.z, self.sp, self.dpdx, self.dpdy, self.Dmin)
        O.interpolate(T, self.U, self.taux, self.tausx)
        O.interpolate(T, self.V, self.tauy, self.tausy)
        if macro_active:
            self.tausxo[...] = self.tausx
            self.tausyo[...] = self.tausy
            self.dpdxo[...] = self.dpdx
            self.dpdyo[...] = self.dpdy
            O.surface_shear_velocity(T, self.taux, self.tauy, self.ustar_s)

    def update_depth(self, _3d=False):
        T, U, V, X = self.T, self.U, self.V, self.X
        if _3d:
            T.zio[...] = T.zin
            T.zin[...] = T.z
            z_T, zo_T = T.zin, T.zio
        else:
            z_T, zo_T = T.z, T.zo
        O.elevation2depth(T, z_T, T.H, -1000.0, T.D)
        np.maximum(T.D, self.Dmin, out=T.Dclip)
        zh = T._work
        np.add(zo_T, z_T, out=zh)
        zh *= 0.5
        for g, mname in ((U, "TU"), (V, "TV"), (X, None)):
            O.interpolate(T, g, zh, g._work)
            if self.ob is not None and mname:
                self.ob.mirror_to(mname, zh, g._work)
            O.elevation2depth(g, g._work, g.H, self.Dmin, g.D)
        with np.errstate(all="ignore"):
            O.alpha(U, U.D, 2 * self.Dmin, self.Dcrit, U.alpha)
            O.alpha(V, V.D, 2 * self.Dmin, self.Dcrit, V.alpha)
        O.elevation2depth(T, zh, T.H, self.Dmin, zh)
        U.ugrid.D[:, :-1] = zh[:, 1:]
        V.vgrid.D[:-1, :] = zh[1:, :]
        U.vgrid.D[:, :] = X.D[1:, 1:]
        V.ugrid.D[:, :] = U.vgrid.D
        if _3d:
            T.ho[...] = T.hn
            U.ho[...] = U.hn
            V.ho[...] = V.hn
            for g, Dc in ((T, T.Dclip), (U, U.D), (V, V.D), (X, X.D)):
                np.multiply(self.dga, Dc, out=g.hn, where=(g.mask != 0)[None])
            for g in (T, U, V):
                O.thickness2vertical_coordinates(g, g.H, g.hn, g.zc, g.zf)
            self.h_T_half[...] = 0.5 * (T.ho + T.hn)
            U.ugrid.hn[:, :, :-1] = self.h_T_half[:, :, 1:]
            V.vgrid.hn[:, :-1, :] = self.h_T_half[:, 1:, :]
            U.vgrid.hn[:, :, :] = X.hn[:, 1:, 1:]
            V.ugrid.hn[:, :, :] = U.vgrid.hn
            if self.runtype == 4:
                O.thickness2center_depth(T, T.hn, self.depth)
