"""Checkpoint/restore of a device-resident simulation: resuming from a
snapshot in a freshly built simulation continues bit for bit like the
uninterrupted run; the reference's restart contract round-trips its fields."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(precision):
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import Simulation

    wl = workloads.seamount(nx=40, ny=30, nz=8, dx=10000.0)
    p = wl.params
    s = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision)
    zc = s.T.zc.all_values
    s.temp.all_values.copy_(torch.where(s.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                        s.temp.all_values.double()))
    s.start(10.0, 7)  # odd split factor: the 2D u/v order does not realign every 3D step
    return s


def _run(s, n3d):
    for _ in range(n3d * s.split_factor):
        s.advance()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_resume_is_bitwise(tmp_path, precision):
    import torch

    from getm_gb300 import checkpoint

    a = _sim(precision)
    _run(a, 3)
    a.advance()  # stop in the middle of a 3D step
    path = str(tmp_path / "snap.npz")
    checkpoint.save(a, path)
    _run(a, 3)
    b = _sim(precision)
    checkpoint.load(b, path)
    _run(b, 3)
    torch.cuda.synchronize()
    sa, sb = checkpoint.state_tensors(a), checkpoint.state_tensors(b)
    assert sa.keys() == sb.keys()
    bad = [k for k in sa if not bool(((sa[k] == sb[k]) | (torch.isnan(sa[k]) & torch.isnan(sb[k]))).all())]
    assert not bad, bad[:10]
    assert a.istep == b.istep


def test_restart_contract(tmp_path):
    import torch

    from getm_gb300 import checkpoint

    a = _sim("fp64")
    _run(a, 2)
    path = str(tmp_path / "restart.npz")
    checkpoint.save_restart(a, path)
    names = set(np.load(path).files)
    assert {"zt", "zot", "zint", "ziot", "hot", "U", "V", "pk", "qk", "Ui", "Vi", "temp", "salt"} <= names
    b = _sim("fp64")
    checkpoint.load_restart(b, path)
    for n, arr in checkpoint.restart_fields(b).items():
        ref = checkpoint.restart_fields(a)[n].all_values
        assert torch.equal(arr.all_values.nan_to_num(), ref.nan_to_num()), n
    np.savez(str(tmp_path / "partial.npz"), zt=np.zeros(1))
    with pytest.raises(Exception, match="part of the model state"):
        checkpoint.load_restart(b, str(tmp_path / "partial.npz"))
