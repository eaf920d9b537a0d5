"""Time-step drivers on the GPU.

``TracerTransport`` runs the tracer-transport configuration: every step is
``TracerCollection.advance`` (python/pygetm/tracer.py:193-276) - the Strang
split u/2, v/2, w, v/2, u/2 of all tracers followed by implicit vertical
diffusion - with prescribed velocities, as in python/tests/test_3d_barotropic.py.
"""

from __future__ import annotations

from typing import Optional

import torch

from .core import CENTERS, INTERFACES, Array, make_grids
from .operators import AdvectionScheme
from .tracer import TracerCollection
from .workloads import Workload


def _dev(a, device):
    return torch.from_numpy(a).to(device=device, dtype=torch.float64).contiguous()


class TracerTransport:
    """Tracer transport through prescribed (u, v, w) with vertical diffusion."""

    def __init__(self, wl: Workload, device="cuda", ntracer: int = 1):
        self.wl = wl
        self.dt = wl.params["dt"]
        self.T = T = make_grids(wl.T, device)
        for g, n in ((T, "T"), (T.ugrid, "U"), (T.vgrid, "V"), (T.xgrid, "X")):
            g.D.all_values.copy_(_dev(wl.fields[f"D_{n}"], device))
            g.hn.all_values.copy_(_dev(wl.fields[f"hn_{n}"], device))
            g.ho = Array(g, g.hn.all_values.clone(), z=CENTERS, name="ho" + g.postfix)
        T.zc.all_values.copy_(_dev(wl.fields["zc_T"], device))
        T.zf.all_values.copy_(_dev(wl.fields["zf_T"], device))
        self.uk = Array(T.ugrid, _dev(wl.fields["uk"], device), z=CENTERS, name="uk")
        self.vk = Array(T.vgrid, _dev(wl.fields["vk"], device), z=CENTERS, name="vk")
        self.w = Array(T, _dev(wl.fields["w"], device), z=INTERFACES, name="ww")
        self.nuh = Array(T, _dev(wl.fields["nuh"], device), z=INTERFACES, name="nuh")
        self.tracers = TracerCollection(T, AdvectionScheme(int(wl.params.get("scheme", 5))), cnpar=wl.params.get("cnpar", 1.0))
        c0 = _dev(wl.fields["tracer"], device)
        for t in range(ntracer):
            tr = self.tracers.add(f"tracer{t}")
            tr.all_values.copy_(c0)

    def step(self):
        self.tracers.advance(self.dt, self.uk, self.vk, self.w, self.nuh)

    def run(self, nstep: int):
        for _ in range(nstep):
            self.step()


# ---------------------------------------------------------------------------
# split-explicit baroclinic simulation
# ---------------------------------------------------------------------------
import enum  # noqa: E402

from . import _lib, _pygetm  # noqa: E402
from .domain import FILL_VALUE, GRAVITY, RHO0  # noqa: E402
from .momentum import CoriolisScheme, Momentum  # noqa: E402
from .operators import AdvectionSplit  # noqa: E402


class RunType(enum.IntEnum):
    """python/pygetm/constants.py:19-23"""

    BAROTROPIC_2D = 1
    BAROTROPIC_3D = 2
    FROZEN_DENSITY = 3
    BAROCLINIC = 4


class Fluxes:
    """Prescribed constant surface fluxes (python/pygetm/airsea.py:109-147)."""

    def __init__(self, taux=0.0, tauy=0.0, sp=101325.0, shf=0.0, swr=0.0, pe=0.0):
        self._ini = dict(taux=taux, tauy=tauy, sp=sp, shf=shf, swr=swr, pe=pe)

    def initialize(self, grid):
        for n, v in self._ini.items():
            a = grid.array(name=n)
            a.fill(v)
            setattr(self, n, a)


class _Split2DPlan:
    """Arguments of the one-launch 2D substep: the fields struct and the
    kernel's barrier words."""

    def __init__(self, fields, sync):
        self.fields = fields
        self.sync = sync


class Simulation:
    """GPU counterpart of pygetm.Simulation (python/pygetm/simulation.py:477-1630)
    for closed domains with prescribed surface fluxes and prescribed vertical
    mixing (``num``/``nuh``), Sigma coordinates, Shchepetkin-McWilliams (or
    Blumberg-Mellor) internal pressure and the device equation of state.

    ``T_host``: HostGrid tree from ``Domain.create_grids(nz, velocity_grids=2)``;
    ``dga``: sigma layer fractions (bottom to surface).
    """

    def __init__(self, T_host, dga, *, runtype: RunType = RunType.BAROCLINIC,
                 advection_scheme: AdvectionScheme = AdvectionScheme.DEFAULT, momentum: Optional[Momentum] = None,
                 airsea: Optional[Fluxes] = None, internal_pressure: str = "shchepetkin_mcwilliams",
                 Dmin: float = 0.02, Dcrit: float = 0.1, delay_slow_ip: bool = False, num: float = 0.0,
                 nuh: float = 0.0, precision: str = "fp64", fused_2d: bool = True, substep_kernel: bool = True,
                 concurrent_3d: bool = True, tiles=None, tracer_storage: Optional[str] = None,
                 internal_pressure_arithmetic: Optional[str] = None, vertical_mixing=None, device="cuda"):
        """``precision``: "fp64" (the plain form) or "mixed" (float32 tracers,
        3D velocities and their tendencies and diffusivities; float64
        elevations, depths, layer thicknesses, 2D transports and their
        accumulation, density, buoyancy, internal pressure and the budget
        sums of ``totals``; increments, tendencies, limiters, drag and the
        internal-pressure slope corrections are evaluated in float).
        ``fused_2d``: the 2D substep's operations run as fused kernels;
        ``substep_kernel``: in addition, a substep that is not followed by a
        3D step runs as one persistent kernel launch (closed domains with the
        default Coriolis scheme, FULL 2D advection split, no horizontal
        momentum diffusion, 3D run types).  ``concurrent_3d``: in a 3D step,
        the shear frequency, the bottom stress, the advection of the 3D
        momentum and the slow terms it feeds run on a second stream,
        concurrently with the tracers, density and internal pressure
        (neither reads what the other writes; the streams join before the
        2D depth update), and the advection of the V momentum on a third,
        beside that of the U momentum; the squared buoyancy frequency joins
        the second stream once the density is known.  ``tiles``: launch
        shapes of the hot kernels (``autotune``): a dict of knob values,
        "auto" for the tuned shapes of this domain's size bucket, or None to
        leave the calling thread's shapes as they are; applied on every
        ``advance`` (and so captured into the step's CUDA graphs).
        ``tracer_storage`` (mixed form): "float64" (the default) keeps the
        tracers (and the buoyancy frequency computed from them) in FP64
        while their advection and diffusion increments, fluxes, limiters and
        solves stay float: float32 rounding of the stored tracers would
        otherwise perturb the density, and through it the flow, by up to half
        an ulp of the tracer every step; "float32" stores them in float.
        ``internal_pressure_arithmetic``: "float32" (mixed-form default: FP64
        column integrals and differences, float slope corrections) or
        "float64".  ``vertical_mixing``: None (prescribed ``num``/``nuh``
        from the arguments of those names) or a
        ``vertical_mixing.VerticalMixing`` instance such as ``GOTM()`` (the
        k-epsilon closure), advanced every 3D step after the 3D momentum
        and before the tracers, as python/pygetm/simulation.py:1107-1115
        does."""
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
        self.precision = precision
        self.fused_2d = fused_2d
        self.substep_kernel = substep_kernel and fused_2d
        self._split2d = None
        self._side_stream = None
        self._forked = False
        d3 = torch.float32 if precision == "mixed" else torch.float64
        self.dtype3d = d3
        if tracer_storage is None:
            tracer_storage = "float64"
        if tracer_storage not in ("float64", "float32"):
            raise ValueError(f"tracer_storage must be 'float64' or 'float32', not {tracer_storage!r}")
        self.tracer_storage = tracer_storage
        if internal_pressure_arithmetic is None:
            internal_pressure_arithmetic = "float32" if precision == "mixed" else "float64"
        self.internal_pressure_arithmetic = internal_pressure_arithmetic
        dtr = torch.float64 if precision == "fp64" or tracer_storage == "float64" else torch.float32
        self.dtype_tracer = dtr
        if Dmin <= 0.0:
            raise Exception("Dmin<=0")
        if Dcrit < 2.5 * Dmin:
            raise Exception("Dcrit < 2.5*Dmin")
        self.runtype = RunType(runtype)
        self.dga = torch.as_tensor(dga, dtype=torch.float64, device=device)[:, None, None]
        self.T = T = make_grids(T_host, device)
        self.U, self.V, self.X = T.ugrid, T.vgrid, T.xgrid
        if precision == "mixed":
            # float metric copies now, ordered after the uploads on this
            # stream (a first use from a kernel would wait for the whole
            # device, every other domain's queued work included)
            for g in T.all_grids():
                g.float_metrics()
        if tiles == "auto":
            from . import autotune

            tiles = autotune.lookup(T.nx, T.ny, T.nz, precision)
        self.tiles = tiles
        self.Dmin, self.Dcrit = Dmin, Dcrit
        self.delay_slow_ip = delay_slow_ip
        three_d = self.runtype > RunType.BAROTROPIC_2D
        T.z = T.array(name="zt")
        T.zo = T.array(name="zot")
        T.z.fill(0.0)
        T.zo.fill(0.0)
        if three_d:
            T.zin = T.array(name="zint")
            T.zio = T.array(name="ziot")
            for g in (T, self.U, self.V):
                g.ho = g.array(name="ho" + g.postfix, z=CENTERS)
        T.Dclip = T.array(name="Dclip")
        if three_d:
            self.h_T_half = T.array(fill=float("nan"), z=CENTERS)
            self.depth = T.array(z=CENTERS, name="pres")
        self.momentum = momentum or Momentum(dtype=d3)
        self.momentum.fused_2d = fused_2d
        # open boundaries (python/pygetm/open_boundaries.py) and model time
        from .open_boundaries import DeviceBoundaries

        ob = getattr(T_host, "open_boundaries", None)
        self._ob = DeviceBoundaries(ob, T, d3) if ob is not None and ob.np > 0 else None
        self.momentum._ob = self._ob
        self._time = torch.zeros((), dtype=torch.float64, device=T.device)
        self.momentum.initialize(T, int(self.runtype), advection_scheme)
        self.airsea = airsea or Fluxes()
        self.airsea.initialize(T)
        self.dpdx = self.U.array(name="dpdx")
        self.dpdy = self.V.array(name="dpdy")
        self.tausx = self.U.array(name="tausxu")
        self.tausy = self.V.array(name="tausyv")
        self.fwf = T.array(name="fwf")
        self.fwf.fill(0.0)
        self.tracers = TracerCollection(T, advection_scheme, dtype=dtr)
        self.vertical_mixing = vertical_mixing
        if three_d and vertical_mixing is not None:
            vertical_mixing.initialize(T, dtype=d3)
            vertical_mixing._ob = self._ob
            self.num, self.nuh = vertical_mixing.num, vertical_mixing.nuh
            # surface roughness for the turbulence closure (simulation.py:777-784)
            self.z0s = T.array(name="z0s")
            self.z0s.fill(0.1)
            self._NN_zero = T.array(z=INTERFACES, name="NN", dtype=d3, fill=0.0)  # without density
        elif three_d:
            self.num = T.array(z=INTERFACES, name="num", dtype=d3)
            self.nuh = T.array(z=INTERFACES, name="nuh", dtype=d3)
            self.num.fill(num)
            self.nuh.fill(nuh)
        if three_d:
            self.ustar_s = T.array(fill=0.0, name="ustar_s")
            self.tausxo = self.U.array(fill_value=None)
            self.tausyo = self.V.array(fill_value=None)
            self.dpdxo = self.U.array(fill_value=None)
            self.dpdyo = self.V.array(fill_value=None)
        self.idpdx = self.idpdy = None
        if self.runtype == RunType.BAROCLINIC:
            self.temp = self.tracers.add("temp", molecular_diffusivity=1.4e-7)
            self.salt = self.tracers.add("salt", molecular_diffusivity=1.1e-9)
            self.temp.fill(5.0)
            self.salt.fill(35.0)
            # density, buoyancy and internal pressure stay float64 in both forms
            self.rho = T.array(z=CENTERS, name="rho")
            self.buoy = T.array(z=CENTERS, name="buoy")
            # squared buoyancy frequency (simulation.py:757-767, :1200-1204)
            self.NN = T.array(z=INTERFACES, name="NN", dtype=d3)
            self.NN.fill(0.0)
            self.internal_pressure_method = internal_pressure
        if three_d:
            # internal_pressure.Base.initialize (python/pygetm/internal_pressure.py:14-30)
            self.idpdx = self.U.array(z=CENTERS, name="idpdx")
            self.idpdy = self.V.array(z=CENTERS, name="idpdy")
            self.idpdx.fill(0.0)
            self.idpdy.fill(0.0)
            self._P_work = torch.zeros((T.nz + 2, T.ny_, T.nx_), dtype=torch.float64, device=T.device)
        self.update_depth(_3d=three_d)
        self.update_depth(_3d=three_d)
        if concurrent_3d and three_d and T.device.type == "cuda":
            self._side_stream = torch.cuda.Stream(device=T.device)
            self.momentum._v_stream = torch.cuda.Stream(device=T.device)

    # ---------------------------------------------------------------- driver
    def start(self, timestep: float, split_factor: int = 1):
        """python/pygetm/simulation.py:207-275"""
        self.timestep = float(timestep)
        self.split_factor = int(split_factor)
        self.macrotimestep = self.timestep * self.split_factor
        self.istep = 0
        self._time.zero_()
        if self._ob is not None:
            self._ob.init_tracer_values(self.tracers._tracers)
        self._start()
        self._update_forcing_and_diagnostics(macro_active=True)
        self._split2d = self._split2d_plan() if self.substep_kernel else None

    def advance(self):
        """python/pygetm/simulation.py:291-325"""
        if self.tiles is not None:
            from . import autotune

            autotune.apply(self.tiles)
        self.istep += 1
        macro_active = self.istep % self.split_factor == 0
        if self._split2d is not None and not macro_active:
            self._split2d_substep()
            return
        _lib.call("getm_advance_time", self._time.data_ptr(), float(self.timestep),
                  torch.cuda.current_stream(self._time.device).cuda_stream)
        self._advance_state(macro_active)
        self._update_forcing_and_diagnostics(macro_active)

    def _split2d_plan(self):
        """Fields of the one-launch 2D substep, or None where that kernel does
        not cover the configuration (the substep then runs operation by
        operation)."""
        m = self.momentum
        if (self._ob is not None or self.runtype <= RunType.BAROTROPIC_2D or m.diffuse_momentum
                or m.An_uu is not None or m.coriolis_scheme != CoriolisScheme.DEFAULT
                or m.advection_split_2d != AdvectionSplit.FULL or not m.uadv.p.value or not m.vadv.p.value
                or self.T.device.type != "cuda"):
            return None
        T, U, V, X, a = self.T, self.U, self.V, self.X, self.airsea
        sync = torch.zeros(4, dtype=torch.int32, device=T.device)  # barrier words, not model state
        fields = _pygetm.split2d_fields(
            mask_t=T.mask, H_t=T.H, iarea_t=T.iarea, z=T.z, zo=T.zo, D_t=T.D, Dclip_t=T.Dclip, work_t=T._work,
            fwf=self.fwf, pe=a.pe, sp=a.sp, taux=a.taux, tauy=a.tauy,
            mask_u=U.mask, H_u=U.H, dy_u=U.dy, idx_u=U.idx, cor_u=U.cor, z0b_u=U.z0b, D_u=U.D, alpha_u=U.alpha,
            work_u=U._work, U=m.U, dpdx=self.dpdx, tausx=self.tausx, corU=m.corU, advU=m.advU, diffU=m.diffU,
            dampU=m.dampU, SxA=m.SxA, SxB=m.SxB, SxD=m.SxD, SxF=m.SxF, ru=m.ru, u1=m.u1, Ucum=m._U_cum,
            advD_u=m.uadv.D, uua=m.uua, uva=m.uva,
            mask_v=V.mask, H_v=V.H, dx_v=V.dx, idy_v=V.idy, cor_v=V.cor, z0b_v=V.z0b, D_v=V.D, alpha_v=V.alpha,
            work_v=V._work, V=m.V, dpdy=self.dpdy, tausy=self.tausy, corV=m.corV, advV=m.advV, diffV=m.diffV,
            dampV=m.dampV, SyA=m.SyA, SyB=m.SyB, SyD=m.SyD, SyF=m.SyF, rv=m.rv, v1=m.v1, Vcum=m._V_cum,
            advD_v=m.vadv.D, vua=m.vua, vva=m.vva,
            mask_x=X.mask, H_x=X.H, D_x=X.D, work_x=X._work, D_uu=U.ugrid.D, D_uv=U.vgrid.D, D_vu=V.ugrid.D,
            D_vv=V.vgrid.D, time=self._time, sync=sync)
        return _Split2DPlan(fields, sync)

    def _split2d_substep(self):
        """A substep without 3D step as one launch (the same operations as
        _advance_state + _update_forcing_and_diagnostics with macro_active
        false, in the same order, with bitwise the same results)."""
        m = self.momentum
        _pygetm.split2d_substep(self._split2d.fields, self.T, self.dtype3d == torch.float32, m._ufirst, True,
                                m.apply_bottom_friction, self.timestep, self.Dmin, self.Dcrit, m.uadv, m.vadv)
        m._ufirst = not m._ufirst

    def split2d_status(self) -> int:
        """Non-zero when a grid barrier of the one-launch substep gave up (the
        substep did not complete; reads the device word)."""
        return 0 if self._split2d is None else int(self._split2d.sync[2].item())

    def clear_split2d_status(self):
        """Re-arm the one-launch substep after a barrier gave up: zero its
        barrier words (stream-ordered, so call it with no substep in flight
        on another stream).  Until then every substep launch returns at once
        and leaves the fields and the model time unchanged."""
        if self._split2d is not None:
            self._split2d.sync.zero_()

    def _start(self):
        """python/pygetm/simulation.py:948-1031"""
        T = self.T
        self.momentum.start()
        for grid in (self.U, self.V):
            edges = grid.water_contact & grid.land
            grid.D.all_values[edges] = FILL_VALUE
            if grid.hn is not None:
                grid.hn.all_values[..., edges] = FILL_VALUE

        minz = -T.H.all_values + self.Dmin

        def clip_z(z):
            shallow = (z.all_values < minz) & T.water
            z.all_values[shallow] = minz[shallow]

        clip_z(T.z)
        clip_z(T.zo)
        three_d = self.runtype > RunType.BAROTROPIC_2D
        if three_d:
            clip_z(T.zin)
            clip_z(T.zio)
        z_backup = T.z.all_values.clone()
        T.z.all_values.copy_(T.zo.all_values)
        self.update_depth(_3d=False)
        if three_d:
            zin_backup = T.zin.all_values.clone()
            T.z.all_values.copy_(T.zio.all_values)
            T.zio.fill(float("nan"))
            T.ho.fill(float("nan"))
            self.update_depth(_3d=True)
            T.z.all_values.copy_(zin_backup)
            self.update_depth(_3d=True, timestep=self.macrotimestep)
            self.momentum.update_diagnostics(self.macrotimestep, self.num)
        T.z.all_values.copy_(z_backup)

    def _advance_state(self, macro_active: bool):
        """python/pygetm/simulation.py:1033-1136"""
        self.momentum.advance_depth_integrated(self.timestep, self.tausx, self.tausy, self.dpdx, self.dpdy)
        self.advance_surface_elevation(self.timestep, self.momentum.U, self.momentum.V, self.fwf)
        if self.runtype > RunType.BAROTROPIC_2D and macro_active:
            # add_freshwater_inputs (simulation.py:1335-1406) is an exact no-op
            # without rivers and with zero precipitation-evaporation.
            self.update_depth(_3d=True, timestep=self.macrotimestep)
            self.momentum.advance(self.macrotimestep, self.split_factor, self.tausxo, self.tausyo, self.dpdxo,
                                  self.dpdyo, self.idpdx, self.idpdy, self.num, side_stream=self._side_stream)
            self._forked = self._side_stream is not None
            if self.vertical_mixing is not None:
                # turbulence from ustar_s, z0s, NN at the start of the step and
                # ustar_b, z0b, SS of the new 3D velocities (simulation.py:1107-1115);
                # SS and ustar_b come from the side stream
                if self._forked:
                    torch.cuda.current_stream(self.T.device).wait_event(self.momentum._bottom_event)
                NN = self.NN if self.runtype == RunType.BAROCLINIC else self._NN_zero
                self.vertical_mixing.advance(self.macrotimestep, self.ustar_s, self.momentum.ustar_b, self.z0s,
                                             self.T.z0b, NN, self.momentum.SS)
            self.tracers.advance(self.macrotimestep, self.momentum.uk, self.momentum.vk, self.momentum.ww, self.nuh)
            if self.runtype == RunType.BAROCLINIC and self.delay_slow_ip:
                _pygetm.column_sums([(self.idpdx, self.momentum.SxB), (self.idpdy, self.momentum.SyB)])

    def _update_forcing_and_diagnostics(self, macro_active: bool):
        """python/pygetm/simulation.py:1138-1304"""
        starting = self.istep == 0
        update_z0b = self.runtype == RunType.BAROTROPIC_2D and not starting
        update_3d = self.runtype > RunType.BAROTROPIC_2D and macro_active
        update_baroclinic = self.runtype == RunType.BAROCLINIC and macro_active
        if update_3d and self._ob is not None:
            # tracers at the open boundaries (simulation.py:1160-1168)
            self._ob.update_tracers(self.tracers._tracers)
        if update_baroclinic:
            self.update_density(side_stream=self._side_stream if self._forked else None)
            self.update_internal_pressure()
            if not self.delay_slow_ip:
                _pygetm.column_sums([(self.idpdx, self.momentum.SxB), (self.idpdy, self.momentum.SyB)])
        if self._forked:  # the momentum advection and slow terms are done
            torch.cuda.current_stream(self.T.device).wait_stream(self._side_stream)
            self._forked = False
        self.update_depth()
        self.momentum.update_depth_integrated_diagnostics(self.timestep, skip_coriolis=not starting,
                                                         update_z0b=update_z0b)
        self.fwf.all_values.copy_(self.airsea.pe.all_values)
        if self._ob is not None:
            # elevation at the open boundaries, before the surface pressure
            # gradient (simulation.py:1252-1257)
            self._ob.prescribe(self._time)
            self._ob.update_elevation(self)
        self.update_surface_pressure_gradient(self.T.z, self.airsea.sp)
        self.airsea.taux.interp(self.tausx)
        self.airsea.tauy.interp(self.tausy)
        if update_3d:
            self.tausxo.all_values.copy_(self.tausx.all_values)
            self.tausyo.all_values.copy_(self.tausy.all_values)
            self.dpdxo.all_values.copy_(self.dpdx.all_values)
            self.dpdyo.all_values.copy_(self.dpdy.all_values)
            _pygetm.surface_shear_velocity(self.airsea.taux, self.airsea.tauy, self.ustar_s)

    # ------------------------------------------------------------ components
    def update_density(self, side_stream=None):
        """density.get_density + buoyancy (simulation.py:1178-1184) and the
        squared buoyancy frequency (:1200-1204) with the device equation of
        state.  ``side_stream``: the squared buoyancy frequency (read by
        nothing else in the step) is issued there; the caller joins it."""
        n = self.rho.all_values.numel()
        from ._lib import call
        from .core import _sfx

        # the mixed form's FP64 tracers: the double-float anomaly from split inputs
        sfx = "_f64s" if self.precision == "mixed" and self.dtype_tracer == torch.float64 else \
            _sfx(self.salt.all_values, self.temp.all_values)
        call("getm_density_buoyancy" + sfx, n, self.salt.all_values.data_ptr(), self.temp.all_values.data_ptr(),
             self.depth.all_values.data_ptr(), self.rho.all_values.data_ptr(), self.buoy.all_values.data_ptr(),
             torch.cuda.current_stream().cuda_stream)
        if side_stream is None:
            _pygetm.buoyancy_frequency(self.salt, self.temp, self.depth, self.NN)
            return
        side_stream.wait_stream(torch.cuda.current_stream(side_stream.device))
        with torch.cuda.stream(side_stream):
            _pygetm.buoyancy_frequency(self.salt, self.temp, self.depth, self.NN)

    def update_internal_pressure(self):
        if self.internal_pressure_method == "blumberg_mellor":
            _pygetm.blumberg_mellor(self.buoy, self.idpdx, self.idpdy)
        else:
            _pygetm.shchepetkin_mcwilliams(self.buoy, self.idpdx, self.idpdy, self._P_work,
                                           self.internal_pressure_arithmetic)

    def totals_device(self) -> torch.Tensor:
        """Device tensor [total volume, total of each tracer] (compensated
        FP64 sums, see ``totals``); no host synchronisation."""
        from ._lib import GETM_TOTALS_BLOCKS, call, ptr_array
        from .core import _sfx

        from ._lib import GETM_MAX_TOTALS

        T = self.T
        trs = list(self.tracers._tracers) if self.runtype > RunType.BAROTROPIC_2D else []
        n = 1 + len(trs)
        chunk = GETM_MAX_TOTALS
        if getattr(self, "_tot_out", None) is None or self._tot_out.numel() != n:
            self._tot_out = torch.zeros(n, dtype=torch.float64, device=T.device)
            self._tot_work = torch.zeros(2 * GETM_TOTALS_BLOCKS * (1 + chunk), dtype=torch.float64, device=T.device)
            self._tot_part = torch.zeros(1 + chunk, dtype=torch.float64, device=T.device)
        hn = T.hn.all_values if trs else T.D.all_values
        groups = [trs[c:c + chunk] for c in range(0, len(trs), chunk)] or [[]]
        for g, grp in enumerate(groups):
            sfx = _sfx(*[t.all_values for t in grp]) if grp else ""
            out = self._tot_out if len(groups) == 1 else self._tot_part
            call("getm_domain_totals" + sfx, T.nx_, T.ny_, max(T.nz, 1), T.halox, T.haloy, T.nx, T.ny,
                 T.mask.all_values.data_ptr(), T.area.all_values.data_ptr(), T.D.all_values.data_ptr(), hn.data_ptr(),
                 len(grp), ptr_array([t.all_values.data_ptr() for t in grp]), self._tot_work.data_ptr(),
                 out.data_ptr(), torch.cuda.current_stream().cuda_stream)
            if len(groups) > 1:
                if g == 0:
                    self._tot_out[0] = self._tot_part[0]
                self._tot_out[1 + g * chunk:1 + g * chunk + len(grp)] = self._tot_part[1:1 + len(grp)]
        return self._tot_out

    @property
    def totals(self):
        """python/pygetm/simulation.py:1409-1444: (total volume, [(tracer,
        total, mean)]) with total volume = sum of D * area and tracer total =
        sum of c * area * hn over the unmasked interior, mean = total / total
        volume.  The sums are compensated (double-double) and reproducible."""
        out = self.totals_device().cpu().tolist()
        trs = list(self.tracers._tracers) if self.runtype > RunType.BAROTROPIC_2D else []
        vol = out[0]
        return vol, [(t, tot, tot / vol) for t, tot in zip(trs, out[1:])]

    def advance_surface_elevation(self, timestep: float, U: Array, V: Array, fwf: Array):
        """simulation.py:1468-1486"""
        if self.fused_2d:
            _pygetm.surface_elevation_fused(timestep, self.T.z, self.T.zo, U, V, fwf)
            return
        self.T.zo.all_values.copy_(self.T.z.all_values)
        _pygetm.advance_surface_elevation(timestep, self.T.z, U, V, fwf)

    def update_surface_pressure_gradient(self, z: Array, sp: Array):
        """simulation.py:1488-1489"""
        _pygetm.surface_pressure_gradient(z, sp, self.dpdx, self.dpdy, self.Dmin,
                                          mixed=self.precision == "mixed")

    def _sigma(self, grid):
        """Sigma.__call__ on one grid (vertical_coordinates.py:106-113)."""
        hn = grid.hn.all_values
        D = grid.Dclip.all_values
        wet = (grid.mask.all_values != 0)
        torch.where(wet, self.dga * D, hn, out=hn)

    def update_depth(self, _3d: bool = False, timestep: float = 0.0):
        """simulation.py:1498-1630"""
        T, U, V, X = self.T, self.U, self.V, self.X
        if _3d:
            T.zio.all_values.copy_(T.zin.all_values)
            T.zin.all_values.copy_(T.z.all_values)
            z_T, zo_T = T.zin, T.zio
        else:
            z_T, zo_T = T.z, T.zo
        if self.fused_2d:
            _pygetm.update_depth_2d(T, z_T, zo_T, self.Dmin, self.Dcrit, mixed=self.precision == "mixed")
        else:
            self._update_depth_2d_ops(z_T, zo_T)
        if self._ob is not None:
            # z_T_half.mirror(z_U), z_T_half.mirror(z_V) (simulation.py:1545-1550)
            self._ob.update_depth(self, z_T, zo_T)
        if _3d:
            self._update_depth_3d()

    def _update_depth_2d_ops(self, z_T, zo_T):
        """The 2D part of update_depth as separate operations."""
        T, U, V, X = self.T, self.U, self.V, self.X
        z_U, z_V, z_X, z_T_half = U._work, V._work, X._work, T._work
        _pygetm.elevation2depth(z_T, T.H, -1000.0, T.D)
        torch.clamp(T.D.all_values, min=self.Dmin, out=T.Dclip.all_values)
        torch.add(zo_T.all_values, z_T.all_values, out=z_T_half.all_values)
        z_T_half.all_values.mul_(0.5)
        z_T_half.interp(z_U)
        _pygetm.elevation2depth(z_U, U.H, self.Dmin, U.D)
        z_T_half.interp(z_V)
        _pygetm.elevation2depth(z_V, V.H, self.Dmin, V.D)
        z_T_half.interp(z_X)
        _pygetm.elevation2depth(z_X, X.H, self.Dmin, X.D)
        _pygetm.alpha(U.D, 2 * self.Dmin, self.Dcrit, U.alpha)
        _pygetm.alpha(V.D, 2 * self.Dmin, self.Dcrit, V.alpha)
        D_T_half = T._work
        _pygetm.elevation2depth(z_T_half, T.H, self.Dmin, D_T_half)
        U.ugrid.D.all_values[:, :-1] = D_T_half.all_values[:, 1:]
        V.vgrid.D.all_values[:-1, :] = D_T_half.all_values[1:, :]
        U.vgrid.D.all_values[:, :] = X.D.all_values[1:, 1:]
        V.ugrid.D.all_values[:, :] = U.vgrid.D.all_values

    def _update_depth_3d(self):
        """The 3D part of update_depth (simulation.py:1588-1630) in one
        launch (getm_update_depth_3d)."""
        if self.fused_2d:
            if getattr(self, "_depth3d", None) is None:
                depth = self.depth if self.runtype == RunType.BAROCLINIC else None
                self._depth3d = _pygetm.depth3d_fields(self.T, self.dga, self.h_T_half, depth)
            _pygetm.update_depth_3d(self._depth3d, self.T)
            return
        self._update_depth_3d_ops()

    def _update_depth_3d_ops(self):
        """The 3D part of update_depth as separate array operations."""
        T, U, V, X = self.T, self.U, self.V, self.X
        T.ho.all_values.copy_(T.hn.all_values)
        U.ho.all_values.copy_(U.hn.all_values)
        V.ho.all_values.copy_(V.hn.all_values)
        for g in (T, U, V, X):
            self._sigma(g)
        for g in (T, U, V):
            _pygetm.thickness2vertical_coordinates(g.mask, g.H, g.hn, g.zc, g.zf)
        torch.add(T.ho.all_values, T.hn.all_values, out=self.h_T_half.all_values)
        self.h_T_half.all_values.mul_(0.5)
        U.ugrid.hn.all_values[:, :, :-1] = self.h_T_half.all_values[:, :, 1:]
        V.vgrid.hn.all_values[:, :-1, :] = self.h_T_half.all_values[:, 1:, :]
        U.vgrid.hn.all_values[:, :, :] = X.hn.all_values[:, 1:, 1:]
        V.ugrid.hn.all_values[:, :, :] = U.vgrid.hn.all_values
        if self.runtype == RunType.BAROCLINIC:
            _pygetm.thickness2center_depth(T.mask, T.hn, self.depth)
