"""The segmented float column solve (GETM_TUNE_COLUMN_SOLVE = 1: four warps
per 32 columns, each owning a quarter of the levels, joined through a reduced
tridiagonal system) against the FP64 oracle and against the
one-thread-per-column sweep.

Both float solves of the mixed form are covered: float storage (the 3D
momentum's viscosity solve, with ea2 and ea4 sources) and FP64 storage (the
tracers, with and without sources), several fields at once (pairs and an odd
last one), the Crank-Nicolson weight 0.5 and 1, old and new thicknesses
different (use_ho), and layer counts where the segments are as short as they
get (8), uneven (13, 30), the benchmark's (40) and at the limit (64); above
it (65) and below 8 the call keeps the one-thread-per-column sweep, bit for
bit.  Tolerances, relative to the largest value (float storage) or change
(FP64 storage): the segmented solve is within twice the error of the
one-thread-per-column sweep (at least 5e-6) of the oracle and of the sweep.
The sweep itself is within 1e-4 here: diffusivities up to 0.1 m2/s over
600 s couple thin layers strongly, and the float solve's rounding grows with
that conditioning (its own tests hold it to 2e-6 at nz = 12).
"""

import numpy as np
import pytest

from tests.gpu_helpers import dev, host
from tests.test_gpu_operators import setup

pytestmark = pytest.mark.gpu


def rel(a, b, mask):
    a = np.asarray(a, dtype=float)[..., mask]
    b = np.asarray(b, dtype=float)[..., mask]
    return float(np.abs(a - b).max() / np.abs(b).max())


def _solve(knob, Td, nuh, fields, mol, ea2, ea4, storage, cnpar, use_ho):
    import torch

    from getm_gb300 import autotune, operators
    from getm_gb300.core import Array, CENTERS, INTERFACES

    autotune.apply({"column_solve": knob})
    try:
        vd = operators.VerticalDiffusion(Td, cnpar)
        dt = torch.float32 if storage == "float32" else torch.float64
        arrs = [Array(Td, dev(f).to(dt), z=CENTERS) for f in fields]
        w32 = lambda a: None if a is None else Array(Td, dev(a).float(), z=CENTERS)  # noqa: E731
        vd.batch(Array(Td, dev(nuh).float(), z=INTERFACES), 600.0, arrs, mol, [w32(e) for e in ea2],
                 [w32(e) for e in ea4], use_ho=use_ho)
        torch.cuda.synchronize()
        return [host(a.all_values).astype(np.float64) for a in arrs]
    finally:
        autotune.apply(None)


def _case(nz, storage, sources, nfields, cnpar, use_ho, seed):
    import oracle.oracle as O

    Th, To, Td, rng = setup(seed=seed, nz=nz)
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    nuh = f32(10.0 ** rng.uniform(-6, -1, (nz + 1, Th.ny_, Th.nx_)))
    base = 0.0 if storage == "float32" else 500.0
    fields = [base + rng.uniform(0, 1, (nz, Th.ny_, Th.nx_)) for _ in range(nfields)]
    if storage == "float32":
        fields = [f32(f) for f in fields]
    mol = [1e-6 * (t + 1) for t in range(nfields)]
    ea2 = [f32(-rng.uniform(0, 1e-2, fields[0].shape)) if sources and t % 2 == 0 else None for t in range(nfields)]
    ea4 = [f32(rng.uniform(0, 1e-3, fields[0].shape)) if sources else None for t in range(nfields)]
    oracle = []
    for t, f in enumerate(fields):
        vo = O.VerticalDiffusion(To, cnpar)
        fo = f.copy()
        vo(nuh, 600.0, fo, molecular=mol[t], ea2=ea2[t], ea4=ea4[t], use_ho=use_ho)
        oracle.append(fo)
    serial = _solve(0, Td, nuh, fields, mol, ea2, ea4, storage, cnpar, use_ho)
    seg = _solve(1, Td, nuh, fields, mol, ea2, ea4, storage, cnpar, use_ho)
    return Th.mask == 1, fields, oracle, serial, seg


def _check(f, o, a, b, wet, storage, label):
    """Errors of both float solves against the oracle: of the values for
    float storage, of the change for FP64 storage (a large mean plus a
    small signal)."""
    if storage == "float64":
        a, b, o = a - f, b - f, o - f
    e_serial, e_seg, e_two = rel(a, o, wet), rel(b, o, wet), rel(b, a, wet)
    print(f"column solve {label}: serial {e_serial:.2e} segmented {e_seg:.2e} between {e_two:.2e}")
    bound = max(2.0 * e_serial, 5e-6)
    assert e_serial < 1e-4   # the one-thread-per-column sweep (conditioning grows with nz and nuh)
    assert e_seg < bound     # the segmented solve: no worse than twice that
    assert e_two < bound


@pytest.mark.parametrize("nz", [8, 13, 30, 40, 64])
@pytest.mark.parametrize("storage,sources", [("float32", True), ("float64", False), ("float64", True)])
def test_segmented_solve_matches_oracle(nz, storage, sources):
    wet, fields, oracle, serial, seg = _case(nz, storage, sources, 3, 1.0, True, seed=500 + nz)
    for t, (f, o, a, b) in enumerate(zip(fields, oracle, serial, seg)):
        _check(f, o, a, b, wet, storage, f"nz={nz} {storage} sources={sources} field {t}")


@pytest.mark.parametrize("cnpar", [0.5, 1.0])
def test_segmented_solve_single_field_same_thickness(cnpar):
    wet, fields, oracle, serial, seg = _case(40, "float64", False, 1, cnpar, False, seed=610)
    _check(fields[0], oracle[0], serial[0], seg[0], wet, "float64", f"nz=40 cnpar={cnpar} ho=hn")


@pytest.mark.parametrize("nz", [4, 65])
def test_outside_the_range_keeps_the_serial_sweep(nz):
    wet, fields, oracle, serial, seg = _case(nz, "float64", True, 2, 1.0, True, seed=700 + nz)
    for a, b in zip(serial, seg):
        assert np.array_equal(a, b)
