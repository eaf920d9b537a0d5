"""Pins the oracle's land masking with the invariant of
python/tests/test_land.py:26-61 (test_nan): every floating-point array of
the simulation is set to NaN on land (mask == 0) before the run starts,
except the grid metrics the reference keeps read-only; after six
baroclinic 3D steps every water point of the prognostic fields is still
finite, so no land value reaches a water point through any operator."""

import numpy as np

from tests.helpers import rotated_pair

# metrics and coordinates: read-only in the reference's test
PROTECTED = {"dx", "dy", "idx", "idy", "area", "iarea", "x", "y", "cor", "H", "z0b_min", "z0b", "zc", "zf"}
# simulation-level arrays by grid
SIM_ARRAYS = {
    "T": ("z", "zo", "zin", "zio", "temp", "salt", "rho", "buoy", "fwf", "sp", "taux", "tauy", "pe", "num", "nuh",
          "depth", "h_T_half", "ustar_s"),
    "U": ("dpdx", "tausx", "idpdx", "tausxo", "dpdxo"),
    "V": ("dpdy", "tausy", "idpdy", "tausyo", "dpdyo"),
}


def _grids(T):
    out, todo = [], [T]
    while todo:
        g = todo.pop()
        if g is None or any(g is o for o in out):
            continue
        out.append(g)
        todo += [g.ugrid, g.vgrid, g.xgrid]
    return out


def test_nan_on_land_never_reaches_water():
    from oracle.models import Simulation

    T0, _, dga = rotated_pair()
    s = Simulation(T0, dga, num=1e-4, nuh=1e-4, taux=0.05)
    T, m = s.T, s.momentum
    s.temp[...] = np.where(T.mask[None] != 0, 10.0 + 0.1 * T.zc, s.temp)
    poisoned = 0
    for g in _grids(T):
        for name, a in list(vars(g).items()):
            if (isinstance(a, np.ndarray) and a.dtype == float and a.ndim >= 2 and name not in PROTECTED
                    and a.shape[-2:] == g.mask.shape):
                a[..., g.mask == 0] = np.nan
                poisoned += 1
    by_grid = {"T": T, "U": T.ugrid, "V": T.vgrid}
    for key, names in SIM_ARRAYS.items():
        for name in names:
            a = getattr(s, name, None)
            if isinstance(a, np.ndarray):
                a[..., by_grid[key].mask == 0] = np.nan
                poisoned += 1
    for name, g in m._grids.items():
        getattr(m, name)[..., g.mask == 0] = np.nan
        poisoned += 1
    assert poisoned > 60
    s.start(10.0, 5)
    for _ in range(30):
        s.advance()
    for name, a, g in (("z", T.z, T), ("temp", s.temp, T), ("salt", s.salt, T), ("U", m.U, T.ugrid),
                       ("V", m.V, T.vgrid), ("uk", m.uk, T.ugrid), ("vk", m.vk, T.vgrid),
                       ("idpdx", s.idpdx, T.ugrid), ("idpdy", s.idpdy, T.vgrid), ("ww", m.ww, T)):
        assert np.isfinite(a[..., g.mask == 1]).all(), name
