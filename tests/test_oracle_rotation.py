"""Pins the oracle's symmetries.

* x/y: the invariant of python/tests/test_rotation.py:28-128: a domain
  rotated by 90 degrees, run with every u/v order reversed (the 2D and 3D
  transports, the momentum advections, the tracer advection), gives the
  rotated fields of the original run.  Four baroclinic 3D steps (20
  substeps) of a closed, stratified domain with random bathymetry and land;
  the reference holds this to 1e-14 (2D) and 1e-12 (3D); the oracle holds it
  to 1e-14 here (measured 4e-16).
* +y/-y: the mirror symmetry that python/tests/test_2d_flow_symmetry.py
  checks for wind-driven flow around an island (there in periodic channels,
  here in a closed domain): the domain mirrored in y, on the f-plane of -f,
  under the same wind along x, gives the mirrored fields (V and vk change
  sign), to 1e-14 (measured 5e-16): upwinding, limiters and staggering treat
  flow in both directions alike."""

import numpy as np

from tests.helpers import mirror_errors, mirrored_pair, rotated_pair, rotation_errors


def _run(T_host, dga, flip, taux=0.0):
    from oracle.models import Simulation

    s = Simulation(T_host, dga, num=1e-4, nuh=1e-4, taux=taux)
    s.temp[...] = np.where(s.T.mask[None] != 0, 10.0 + 0.1 * s.T.zc, s.temp)
    s.start(10.0, 5)
    if flip:  # test_rotation.py:62-66
        m = s.momentum
        m._ufirst, m._u3dfirst = not m._ufirst, not m._u3dfirst
        m.uadv.ufirst, m.vadv.ufirst = not m.uadv.ufirst, not m.vadv.ufirst
        s.adv.ufirst = not s.adv.ufirst
    for _ in range(20):
        s.advance()
    m = s.momentum
    return s, {"z": s.T.z, "temp": s.temp, "U": m.U, "V": m.V, "uk": m.uk, "vk": m.vk}


def test_rotated_domain_gives_the_rotated_fields():
    T0, Tr, dga = rotated_pair()
    _, orig = _run(T0, dga, False)
    s, rot = _run(Tr, dga, True)
    errs = rotation_errors(orig, rot, (s.T.mask, s.T.ugrid.mask, s.T.vgrid.mask))
    assert max(errs.values()) < 1e-14, errs
    # and the flow is not trivial
    assert np.abs(orig["U"]).max() > 1e-6 and np.abs(orig["uk"]).max() > 1e-7


def test_mirrored_domain_gives_the_mirrored_fields():
    T0, Tm, dga = mirrored_pair()
    _, orig = _run(T0, dga, False, taux=0.05)
    s, mir = _run(Tm, dga, False, taux=0.05)
    errs = mirror_errors(orig, mir, (s.T.mask, s.T.ugrid.mask, s.T.vgrid.mask))
    assert max(errs.values()) < 1e-14, errs
    assert np.abs(orig["U"]).max() > 1e-3 and np.abs(orig["V"]).max() > 1e-4
