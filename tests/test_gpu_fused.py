"""Fused 2D-substep kernels: with FP64 arithmetic the fused sequences give
bitwise the same state as the separate operations; in the mixed form (float
increments) the error against FP64 stays that of the unfused mixed path."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _seamount(precision, fused, n3d=3):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount(nx=40, ny=30, nz=8, dx=10000.0)
    p = wl.params
    s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, fused_2d=fused)
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                        s.temp.all_values.double()).float().double())
    s.start(10.0, 7)
    for _ in range(n3d * 7 + 3):
        s.advance()
    torch.cuda.synchronize()
    return s


def test_fused_fp64_is_bitwise():
    import torch

    from getm_gb300 import checkpoint

    a, b = _seamount("fp64", True), _seamount("fp64", False)
    sa, sb = checkpoint.state_tensors(a), checkpoint.state_tensors(b)
    bad = [k for k in sa if not bool(((sa[k] == sb[k]) | (torch.isnan(sa[k]) & torch.isnan(sb[k]))).all())]
    assert not bad, bad[:12]


def _member(precision, fused, n3d=4):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.ensemble import make_member

    wl = workloads.ensemble_member(np.random.default_rng(3), nmin=40, nmax=48, nzmin=6, nzmax=8)
    s = make_member(wl, precision)
    s.fused_2d = s.momentum.fused_2d = fused
    for _ in range(n3d * s.split_factor):
        s.advance()
    torch.cuda.synchronize()
    return s


def test_fused_mixed_error_vs_fp64():
    """A wind-driven member (real currents): the mixed form's elevation and
    transport errors against FP64 with the fused kernels are within a factor
    two of those of the separate operations."""
    from tests.gpu_helpers import host

    ref = _member("fp64", True)
    wet = ref.T.mask.all_values.cpu().numpy() == 1
    uwet = ref.U.mask.all_values.cpu().numpy() == 1

    def err(s):
        z = np.abs(host(s.T.z.all_values) - host(ref.T.z.all_values))[wet].max()
        U = np.abs(host(s.momentum.U.all_values) - host(ref.momentum.U.all_values))[uwet].max()
        return z, U

    zf, Uf = err(_member("mixed", True))
    zu, Uu = err(_member("mixed", False))
    zmax = np.abs(host(ref.T.z.all_values))[wet].max()
    Umax = np.abs(host(ref.momentum.U.all_values))[uwet].max()
    print(f"mixed vs fp64: fused z {zf / zmax:.2e} U {Uf / Umax:.2e}; separate z {zu / zmax:.2e} U {Uu / Umax:.2e}")
    assert zf <= 2 * zu + 1e-6 * zmax
    assert Uf <= 2 * Uu + 1e-6 * Umax
