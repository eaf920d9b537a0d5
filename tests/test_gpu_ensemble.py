"""Batched ensemble: every member's result is the same alone and in the mix
(bit for bit: the same kernels run on the same inputs; members share no
state), and the graph replay matches eager stepping."""

import pytest

pytestmark = pytest.mark.gpu


def _members(n=3, seed=11):
    import numpy as np

    from getm_gb300 import workloads

    rng = np.random.default_rng(seed)
    return [workloads.ensemble_member(rng, nmin=24, nmax=40, nzmin=5, nzmax=8) for _ in range(n)]


def _differences(a, b):
    """Points where a and b differ (NaN equals NaN)."""
    import torch

    diff = ~((a == b) | (torch.isnan(a) & torch.isnan(b)))
    return int(diff.sum()), diff.nonzero()[:4].tolist()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_in_mix(precision):
    import torch

    from getm_gb300.ensemble import Ensemble, make_member

    wls = _members()
    ens = Ensemble([make_member(w, precision) for w in wls], lanes=2)
    ens.prepare()  # 2 eager warm-up steps; capture runs nothing
    for _ in range(3):
        ens.step()
    torch.cuda.synchronize()
    bad = []
    for n, (w, m) in enumerate(zip(wls, ens.members)):
        alone = make_member(w, precision)
        for _ in range(5 * alone.split_factor):  # 2 warm-up + 3 replayed steps, eagerly
            alone.advance()
        torch.cuda.synchronize()
        fields = {"temp": (alone.temp, m.temp), "salt": (alone.salt, m.salt), "z": (alone.T.z, m.T.z),
                  "U": (alone.momentum.U, m.momentum.U), "uk": (alone.momentum.uk, m.momentum.uk)}
        for name, (x, y) in fields.items():
            count, where = _differences(x.all_values, y.all_values)
            if count:
                bad.append(f"member {n} {name}: {count} points differ, e.g. {where}")
    assert not bad, "\n".join(bad)


def test_sequential_equals_concurrent():
    """Replaying the members one after another on one stream gives the same
    results as the lane-concurrent replay."""
    import torch

    from getm_gb300.ensemble import Ensemble, make_member

    wls = _members(n=2, seed=12)
    a = Ensemble([make_member(w, "mixed") for w in wls], lanes=2)
    b = Ensemble([make_member(w, "mixed") for w in wls], lanes=2)
    a.prepare()
    b.prepare()
    for _ in range(2):
        a.step()
        b.step(sequential=True)
    torch.cuda.synchronize()
    for x, y in zip(a.members, b.members):
        assert _differences(x.temp.all_values, y.temp.all_values)[0] == 0
        assert _differences(x.T.z.all_values, y.T.z.all_values)[0] == 0
