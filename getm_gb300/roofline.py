"""Algorithmic bytes of one split-explicit 3D step (the HBM roofline's
numerator for the whole step).

Rule: per call at pygetm's operator API (python/_pygetm.pyx and the numpy
array operations of python/pygetm/{simulation,momentum,tracer}.py), every
distinct 3D operand counts once read and every output once written, at the
storage precision of the form; 2D operands count per water column; work
arrays a kernel keeps to itself (fluxes, Thomas coefficients) do not count.
Interior cells only (nx ny nz; columns nx ny), halos excluded.

Storage: the FP64 form stores everything in 8 bytes.  The mixed form
stores 3D velocities and transports and their tendencies, diffusivities, w
and the shear frequency in 4 bytes, the tracers and the buoyancy frequency
in 8 bytes (4 with ``tracer_storage="float32"``), and keeps layer
thicknesses, vertical coordinates, density, buoyancy, the internal-pressure
gradients and every 2D field in 8 bytes.

The call list follows Simulation.advance for a closed baroclinic domain
with prescribed surface fluxes and vertical mixing, default Coriolis, FULL
2D advection split and no horizontal momentum diffusion (the seamount
box): ``split`` substeps, the last of which also runs the 3D step.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, List

D = 8  # float64
M = 4  # int32 mask


@dataclasses.dataclass
class Call:
    name: str          # operator call (reference file:line)
    per_cell: float    # 3D bytes per interior cell
    per_column: float  # 2D bytes per interior column
    count: int = 1     # calls per 3D step


def _transport_2d_momentum() -> float:
    """_transport_2d_momentum (momentum.py:1017-1097), bytes per column:
    u1 = U/D, v1 = V/D; bottom friction (two interps, two drag coefficients
    from mask, u, v, D, z0b); per direction two interps to the advection
    grids, two divisions, the copy into advU, the FULL split (D work copy and
    two u_2d/v_2d passes: u, hu, h, var in; h, var out) and
    reconstruct_transport_change (var, D, U in; var out)."""
    per_dir = 2 * 2 * D + 2 * 3 * D + 2 * D + (2 * D + 2 * 6 * D) + 4 * D
    return 2 * 3 * D + 2 * 2 * D + 2 * (M + 4 * D + D) + 2 * per_dir


def _substep_2d() -> List[Call]:
    """The 2D operations of one substep (every substep), bytes per column."""
    c = []
    # advance_2d_transport, U then V (momentum.F90:147-189): reads mask,
    # alpha, D, dp, taus, cor, adv, diff, damp, SA, SB, SD, SF, r and U;
    # writes U
    c.append(Call("advance_2d_transport x2 (momentum.F90:147-189)", 0, 2 * (M + 14 * D + D)))
    # coriolis U -> V and V -> U (momentum.py:1127-1148): transport, f in; term out
    c.append(Call("coriolis 2D x2 (momentum.py:1127-1148)", 0, 2 * 3 * D))
    # _U_cum += U, _V_cum += V (momentum.py:716-718)
    c.append(Call("accumulate transports (momentum.py:716-718)", 0, 6 * D))
    # zo = z; advance_surface_elevation (wrapper.F90:496-523): mask, z, U, V,
    # fwf, dyu, dxv, iarea in; z out
    c.append(Call("surface elevation (simulation.py:1468-1486, wrapper.F90:496-523)", 0, 2 * D + M + 8 * D))
    # update_depth, 2D part (simulation.py:1498-1586): elevation2depth on T
    # (z, H, mask -> D), Dclip, z_T_half, interp to U/V/X and elevation2depth
    # on each, alpha on U and V, D_T_half, four depth copies UU/VV/UV/VU
    e2d = 3 * D + M
    c.append(Call("update_depth 2D (simulation.py:1498-1586)", 0,
                  e2d + 2 * D + 3 * D + 3 * (2 * D + e2d) + 2 * (2 * D + M) + e2d + 4 * 2 * D))
    c.append(Call("_transport_2d_momentum (momentum.py:1017-1097)", 0, _transport_2d_momentum()))
    # surface_pressure_gradient (wrapper.F90:525-565): z, sp, H, D, idx, mask in; dpdx out (x and y)
    c.append(Call("surface_pressure_gradient (wrapper.F90:525-565)", 0, 2 * (5 * D + M + D)))
    # wind stress interpolation to U and V, fwf = pe (simulation.py:1216-1280)
    c.append(Call("stress interp + fwf (simulation.py:1216-1280)", 0, 3 * 2 * D))
    return c


def step_calls(precision: str = "mixed", ntracer: int = 2, split: int = 30,
               tracer_storage: str = "float64") -> List[Call]:
    """Every call of one 3D step with its substeps, for the given form."""
    if precision not in ("fp64", "mixed") or tracer_storage not in ("float64", "float32"):
        raise ValueError((precision, tracer_storage))
    S = 4 if precision == "mixed" else 8  # bytes of a float-stored 3D field
    F = 4 if precision == "mixed" and tracer_storage == "float32" else 8  # bytes of a tracer
    H = D                                 # thicknesses, coordinates: float64 in both forms
    calls = [dataclasses.replace(c, count=split) for c in _substep_2d()]
    # --- 3D step (macro substep) ---
    # update_depth(_3d=True) (simulation.py:1588-1630): ho <- hn on T, U, V;
    # Sigma hn = dga D on T, U, V, X; thickness2vertical_coordinates on T, U, V
    # (hn in; zc, zf out); h_T_half; UU/VV/UV/VU thickness copies; centre depth
    calls.append(Call("update_depth 3D (simulation.py:1588-1630)",
                      3 * 2 * H + 4 * H + 3 * 3 * H + 3 * H + 4 * 2 * H + 2 * H, 4 * D))
    # Momentum.advance, per direction (momentum.py:1164-1214):
    # collect_3d_momentum_sources (ho, hn, cor, adv, diff, idp in; ea4 out),
    # viscosity interp, implicit vertical viscosity (visc, ho, hn, vel, ea2,
    # ea4 in; vel out), tp3d = vel hn, its column sum and correction, 3D Coriolis
    per_dir = ((2 * H + 3 * S + D + S) + 2 * S + (S + 2 * H + 3 * S + S) + (S + H + S) + S + (S + H + S) + 2 * S)
    calls.append(Call("Momentum.advance x2 directions (momentum.py:760-858, 1164-1214)", 2 * per_dir,
                      2 * (5 * D + M) + 5 * D))
    # update_diagnostics (momentum.py:860-1015): w_momentum_3d (pk, qk, ho,
    # hn in; w out), uk and vk, shear_frequency (uk, vk, hnU, hnV in; SS
    # out), per direction the advected copy, three interps (two velocities,
    # w), apply_3d (four u/v passes of var, u, hu, h in and h, var out; the w
    # pass of w, h, var in and h, var out) and reconstruct_transport_change;
    # the column sums of advpk, advqk, diffpk, diffqk
    def apply3d_of(f):  # f: bytes of the advected field
        return 4 * (f + S + H + H + H + f) + (S + H + f + H + f)

    apply3d = apply3d_of(S)
    adv_dir = 2 * S + 3 * 2 * S + apply3d + (S + H + S + S)
    # 2D: bottom friction on the bottom layer (two interps, two drag
    # coefficients), bottom_shear_velocity (three masks, u, v, rru, rrv in;
    # ustar2_x, ustar2_y, ustar out), _transport_2d_momentum of Ui and Vi,
    # SxF and SyF (ustar2, r, u1 in; SxF out)
    calls.append(Call("Momentum.update_diagnostics (momentum.py:860-1015)",
                      (2 * S + 2 * H + S) + 2 * (S + H + S) + (2 * S + 2 * H + S) + 2 * adv_dir + 4 * S,
                      2 * 2 * D + 2 * (M + 4 * D + D) + (3 * M + 7 * D) + _transport_2d_momentum() + 2 * 4 * D))
    # TracerCollection.advance (tracer.py:193-276): per tracer apply_3d (as
    # above with float u/v/w) and VerticalDiffusion (nuh, ho, hn, var in; var out)
    calls.append(Call("TracerCollection.advance (tracer.py:193-276)",
                      ntracer * (apply3d_of(F) + (S + 2 * H + F + F)), 0))
    # density and buoyancy (simulation.py:1178-1184): S, T, pressure in; rho,
    # then buoy; internal pressure (buoy, h, zc in; idpdx, idpdy out);
    # SxB, SyB column sums; NN (S, T, h, pressure in; NN out)
    calls.append(Call("density, buoyancy, internal pressure, NN (simulation.py:1178-1204)",
                      (2 * F + H + D) + 2 * D + 5 * D + 2 * D + (2 * F + 2 * H + F), 2 * D))
    return calls


def step_bytes(nx: int, ny: int, nz: int, precision: str = "mixed", ntracer: int = 2,
               split: int = 30, tracer_storage: str = "float64") -> Dict[str, float]:
    """Algorithmic bytes of one 3D step: per call and in total, with the 2D
    substep loop and the 3D part apart."""
    cells, cols = nx * ny * nz, nx * ny
    out: Dict[str, float] = {}
    b2d = b3d = 0.0
    for c in step_calls(precision, ntracer, split, tracer_storage):
        b = c.count * (c.per_cell * cells + c.per_column * cols)
        out[c.name] = b
        if c.per_cell:
            b3d += c.count * c.per_cell * cells
        b2d += c.count * c.per_column * cols
    out["total"] = b2d + b3d
    out["3d"] = b3d
    out["2d"] = b2d
    return out


def substep_bytes(nx: int, ny: int) -> float:
    """Algorithmic bytes of one 2D substep without 3D step."""
    return sum(c.per_column for c in _substep_2d()) * nx * ny
