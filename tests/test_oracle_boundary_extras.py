"""Oracle restatements of the three remaining boundary entries
(python/_pygetm.pyx:468-479, 574-585): properties the reference routines
guarantee, checked on the CPU."""

import numpy as np

import oracle.oracle as O
from getm_gb300.domain import calculate_sigma


def test_vertical_advection_to_sources_conserves_and_idles():
    rng = np.random.default_rng(3)
    nz, ny, nx = 6, 9, 11
    mask = np.ones((nz, ny, nx), dtype=np.int32)
    mask[:, 4, 5] = 0
    c = rng.uniform(0.5, 2.0, (nz, ny, nx))
    h = rng.uniform(1.0, 3.0, (nz, ny, nx))
    w = rng.uniform(-1e-3, 1e-3, (nz, ny, nx))
    s = np.zeros((nz, ny, nx))
    O.vertical_advection_to_sources(2, 2, mask, c, w, h, s)
    # what leaves one level enters the next: the column integral of s h is 0
    assert np.abs((s * h).sum(axis=0)).max() < 1e-18
    assert np.abs(s[:, 2:-2, 2:-2]).max() > 0 and (s[:, :2] == 0).all() and (s[:, 4, 5] == 0).all()
    # w zero at every interior point: nothing changes, NaN in c included
    c[0, 3, 3] = np.nan
    s2 = rng.uniform(size=s.shape)
    before = s2.copy()
    w2 = np.zeros_like(w)
    w2[:, 0, :] = 1.0  # halo only
    O.vertical_advection_to_sources(2, 2, mask, c, w2, h, s2)
    assert np.array_equal(s2, before)


def test_update_gvc_reference_layer():
    nz, ny, nx = 10, 5, 6
    dbeta = calculate_sigma(nz, 1.5, 1.0)
    dsigma = 1.0 / nz
    D = np.linspace(5.0, 200.0, ny * nx).reshape(ny, nx)
    mask = np.ones((ny, nx), dtype=np.int32)
    mask[0, 0] = 0
    h = np.full((nz, ny, nx), -1.0)
    Dgamma = 40.0
    O.update_gvc(dsigma, dbeta, Dgamma, -1, D, mask, h)
    wet = mask == 1
    np.testing.assert_allclose(h[-1][wet], (np.minimum(Dgamma, D) * dsigma)[wet], rtol=1e-12)
    np.testing.assert_allclose(h.sum(axis=0)[wet], D[wet], rtol=1e-12)
    assert (h[:, 0, 0] == -1.0).all()
