"""Batched ensemble: every member's result is the same alone and in the mix
(bit for bit: the same kernels run on the same inputs; members share no
state), and the graph replay matches eager stepping."""

import pytest

pytestmark = pytest.mark.gpu


def _members(n=3, seed=11):
    from getm_gb300 import workloads

    import numpy as np

    rng = np.random.default_rng(seed)
    return [workloads.ensemble_member(rng, nmin=24, nmax=40, nzmin=5, nzmax=8) for _ in range(n)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_in_mix(precision):
    import torch

    from getm_gb300.ensemble import Ensemble, make_member

    wls = _members()
    ens = Ensemble([make_member(w, precision) for w in wls])
    ens.warmup(1)
    ens.capture()
    for _ in range(2):
        ens.step_period()
    torch.cuda.synchronize()
    nsteps = {id(m): m for m in ens.members}
    for w, m in zip(wls, ens.members):
        alone = make_member(w, precision)
        # warm-up period + capture period + 2 replays = 4 periods of 2 3D steps
        for _ in range(4 * Ensemble.period * alone.split_factor):
            alone.advance()
        torch.cuda.synchronize()
        for name in ("temp", "salt"):
            assert torch.equal(getattr(alone, name).all_values, getattr(m, name).all_values), name
        assert torch.equal(alone.T.z.all_values, m.T.z.all_values)
        assert torch.equal(alone.momentum.U.all_values, m.momentum.U.all_values)
        assert torch.equal(alone.momentum.uk.all_values, m.momentum.uk.all_values)
    del nsteps
