"""The elimination of the segmented column solve (vd_seg_kernel,
getm_gb300/csrc/vertical_diffusion.cu) restated step for step in numpy and
checked against a direct solve: the partition method for tridiagonal
systems (Wang 1981) with four segments per column.  Each segment eliminates
its rows in terms of its first and last unknowns (forward, then backward),
contributes two rows to a reduced system of eight unknowns solved by Thomas
elimination, and substitutes back.  Diagonally dominant systems like the
implicit diffusion's, every layer count the kernel takes (8..64, uneven
segments included), agreement to 1e-13 relative."""

import numpy as np
import pytest

NSEG = 4


def partition_solve(lw, dg, up, rh):
    """lw[k] x[k-1] + dg[k] x[k] + up[k] x[k+1] = rh[k] (lw[0] = up[-1] = 0)."""
    nz = len(dg)
    R = 2 * NSEG
    red = np.zeros((4, R))
    segs = []
    for s in range(NSEG):
        klo = s * nz // NSEG
        m = (s + 1) * nz // NSEG - klo
        rows = {}
        for ii in range(m):
            k = klo + ii
            if ii == 0:
                L0, D0, U0, R0 = lw[k], dg[k], up[k], rh[k]
            elif ii == 1:
                inv = 1.0 / dg[k]
                al, ga, de = lw[k] * inv, up[k] * inv, rh[k] * inv
            else:
                inv = 1.0 / (dg[k] - lw[k] * ga)
                al, ga, de = -(lw[k] * al) * inv, up[k] * inv, (rh[k] - lw[k] * de) * inv
            if 1 <= ii < m - 1:
                rows[ii] = [al, ga, de]
        as_, gs, ds = 0.0, -1.0, 0.0
        for ii in range(m - 2, 0, -1):
            a_, g_, d_ = rows[ii]
            ds, as_, gs = d_ - g_ * ds, a_ - g_ * as_, -(g_ * gs)
            rows[ii] = [as_, gs, ds]
        red[:, 2 * s] = [L0, D0 - U0 * as_, -(U0 * gs), R0 - U0 * ds]
        red[:, 2 * s + 1] = [al, 1.0, ga, de]
        segs.append((klo, m, rows))
    cp, dp = np.zeros(R), np.zeros(R)
    cp[0], dp[0] = red[2, 0] / red[1, 0], red[3, 0] / red[1, 0]
    for r in range(1, R):
        inv = 1.0 / (red[1, r] - red[0, r] * cp[r - 1])
        cp[r], dp[r] = red[2, r] * inv, (red[3, r] - red[0, r] * dp[r - 1]) * inv
    x = np.zeros(R)
    x[-1] = dp[-1]
    for r in range(R - 2, -1, -1):
        x[r] = dp[r] - cp[r] * x[r + 1]
    out = np.zeros(nz)
    for s, (klo, m, rows) in enumerate(segs):
        xF, xL = x[2 * s], x[2 * s + 1]
        for ii in range(m):
            out[klo + ii] = xF if ii == 0 else xL if ii == m - 1 else rows[ii][2] - rows[ii][0] * xF - rows[ii][1] * xL
    return out


@pytest.mark.parametrize("nz", [8, 9, 10, 13, 20, 30, 40, 41, 63, 64])
def test_partition_solve_matches_a_direct_solve(nz):
    rng = np.random.default_rng(nz)
    for _ in range(5):
        an = 10.0 ** rng.uniform(-3, 2, nz + 1)  # coupling of each interface
        an[0] = an[-1] = 0.0
        h = rng.uniform(0.1, 3.0, nz)
        lw, up = -an[:nz], -an[1:]
        dg = h + an[:nz] + an[1:]
        rh = rng.normal(size=nz)
        A = np.diag(dg) + np.diag(lw[1:], -1) + np.diag(up[:-1], 1)
        direct = np.linalg.solve(A, rh)
        x = partition_solve(lw, dg, up, rh)
        assert np.abs(x - direct).max() / np.abs(direct).max() < 1e-13
