"""The invariant of python/tests/test_rotation.py:28-128 on the GPU: the FP64
split-explicit step (one-launch 2D substeps, fused 3D step) on a domain
rotated by 90 degrees, with every u/v order reversed, gives the rotated
fields of the original run.  x and y run through different kernels here
(warp-shuffle x passes, marching y passes, transposed tiles in the substep),
so this checks that they compute the same thing.  The reference holds it to
1e-12 for 3D runs, and so does this test."""

import numpy as np
import pytest

from tests.helpers import rotated_pair, rotation_errors

pytestmark = pytest.mark.gpu


def _run(T_host, dga, flip):
    import torch

    from getm_gb300.simulation import Simulation

    s = Simulation(T_host, dga, num=1e-4, nuh=1e-4, device="cuda:0")
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 10.0 + 0.1 * zc, s.temp.all_values))
    s.start(10.0, 5)
    if flip:
        m = s.momentum
        m._ufirst, m._u3dfirst = not m._ufirst, not m._u3dfirst
        m.uadv.ufirst, m.vadv.ufirst = not m.uadv.ufirst, not m.vadv.ufirst
        s.tracers._advection.ufirst = not s.tracers._advection.ufirst
    for _ in range(20):
        s.advance()
    torch.cuda.synchronize()
    assert s.split2d_status() == 0
    m = s.momentum
    host = lambda a: a.all_values.double().cpu().numpy()  # noqa: E731
    return s, {"z": host(s.T.z), "temp": host(s.temp), "U": host(m.U), "V": host(m.V), "uk": host(m.uk),
               "vk": host(m.vk)}


def test_rotated_domain_gives_the_rotated_fields():
    T0, Tr, dga = rotated_pair()
    _, orig = _run(T0, dga, False)
    s, rot = _run(Tr, dga, True)
    masks = tuple(g.mask.all_values.cpu().numpy() for g in (s.T, s.T.ugrid, s.T.vgrid))
    errs = rotation_errors(orig, rot, masks)
    print("rotation errors", errs)
    assert max(errs.values()) < 1e-12, errs
    assert np.abs(orig["U"]).max() > 1e-6 and np.abs(orig["uk"]).max() > 1e-7
