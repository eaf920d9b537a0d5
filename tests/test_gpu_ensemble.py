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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_substeps_equal_alone(precision):
    """Members of uneven size and substep count advanced with every plain 2D
    substep of all members in one cooperative launch per substep index
    (getm_substep_batch_launch), graph-replayed rounds: each member's state
    is bitwise that of the member advanced alone (its own one-launch
    substeps), also at an odd number of rounds."""
    import torch

    from getm_gb300.ensemble import BatchedEnsemble, make_member

    wls = _members(n=4, seed=13)
    splits = sorted({w.params["split_factor"] for w in wls})
    ens = BatchedEnsemble([make_member(w, precision, substep_kernel=True) for w in wls], lanes=3)
    ens.prepare()  # 2 warm-up rounds member by member; capture runs nothing
    for _ in range(3):
        ens.step()
    torch.cuda.synchronize()
    assert ens.status() == 0
    bad = []
    for n, (w, m) in enumerate(zip(wls, ens.members)):
        alone = make_member(w, precision, substep_kernel=True)
        for _ in range(5 * alone.split_factor):
            alone.advance()
        torch.cuda.synchronize()
        fields = {"temp": (alone.temp, m.temp), "z": (alone.T.z, m.T.z), "U": (alone.momentum.U, m.momentum.U),
                  "V": (alone.momentum.V, m.momentum.V), "uk": (alone.momentum.uk, m.momentum.uk),
                  "time": (alone._time, m._time)}
        for name, (x, y) in fields.items():
            xv = x if isinstance(x, torch.Tensor) else x.all_values
            yv = y if isinstance(y, torch.Tensor) else y.all_values
            count, where = _differences(xv, yv)
            if count:
                bad.append(f"member {n} (split {w.params['split_factor']}) {name}: {count} points differ, e.g. {where}")
    assert not bad, f"splits {splits}\n" + "\n".join(bad)


def test_batched_eager_equals_graphs():
    """The batched rounds issued eagerly equal their graph replay."""
    import torch

    from getm_gb300.ensemble import BatchedEnsemble, make_member

    wls = _members(n=3, seed=14)
    a = BatchedEnsemble([make_member(w, "mixed", substep_kernel=True) for w in wls], lanes=2)
    b = BatchedEnsemble([make_member(w, "mixed", substep_kernel=True) for w in wls], lanes=2)
    a.prepare()
    for s in b.members:  # the same warm-up, then eager rounds
        for _ in range(2 * s.split_factor):
            s.advance()
    torch.cuda.synchronize()
    b._register()
    for _ in range(3):
        a.step()
        b.step()
    torch.cuda.synchronize()
    assert a.status() == 0 and b.status() == 0
    for x, y in zip(a.members, b.members):
        assert _differences(x.temp.all_values, y.temp.all_values)[0] == 0
        assert _differences(x.momentum.U.all_values, y.momentum.U.all_values)[0] == 0
