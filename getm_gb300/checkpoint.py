"""Checkpoint and restore of device-resident simulations.

Two levels:

* ``checkpoint``/``restore``: a snapshot of the complete device state of a
  ``Simulation`` (every tensor reachable from the simulation, its momentum,
  tracers, surface forcing and grid tree) plus the host-side counters that
  select the next step's code path (step index, the u/v orders of the 2D and
  3D momentum updates).  Restoring a snapshot into a simulation built from
  the same workload and continuing gives results bit for bit equal to an
  uninterrupted run: a domain can be paused, evicted from HBM and resumed.
  ``save``/``load`` write the snapshot to an ``.npz`` file.

* ``save_restart``/``load_restart``: the reference's restart contract
  (python/pygetm/simulation.py:128-202 load_restart and
  python/pygetm/output/__init__.py:207-225 add_restart): the fields flagged
  ``_part_of_state`` in the reference, under the reference's names, written
  before a run ends and loaded before ``start``; ``start`` then rebuilds every
  diagnostic from them, as pygetm does.
"""

from __future__ import annotations

from typing import Dict, Iterator, Tuple

import numpy as np
import torch

from .core import Array, Grid

# host attributes that decide the next step's code path
_HOST_COUNTERS = {
    "sim": ("istep", "timestep", "split_factor", "macrotimestep"),
    "momentum": ("_ufirst", "_u3dfirst"),
}


def _tensors_of(obj, prefix: str, seen: set) -> Iterator[Tuple[str, torch.Tensor]]:
    for name, val in sorted(vars(obj).items()):
        if isinstance(val, Array):
            t = val.all_values
        elif isinstance(val, torch.Tensor):
            t = val
        else:
            continue
        key = (t.data_ptr(), t.dtype, tuple(t.shape), t.stride())
        if key in seen or t.numel() == 0:
            continue
        seen.add(key)
        yield f"{prefix}{name}", t


def state_tensors(sim) -> Dict[str, torch.Tensor]:
    """Every device tensor that can carry state between steps, by a stable
    qualified name (views of a tensor already listed are skipped)."""
    seen: set = set()
    out: Dict[str, torch.Tensor] = {}
    for g in sim.T.all_grids():
        for k, t in _tensors_of(g, f"grid{g.postfix or 't'}.", seen):
            out[k] = t
    objs = [("sim.", sim), ("momentum.", sim.momentum), ("airsea.", sim.airsea)]
    if getattr(sim, "vertical_mixing", None) is not None:
        objs.append(("vertical_mixing.", sim.vertical_mixing))
    for prefix, obj in objs:
        for k, t in _tensors_of(obj, prefix, seen):
            out[k] = t
    for tr in sim.tracers._tracers:
        for k, t in _tensors_of_tracer(tr, seen):
            out[k] = t
    return out


def _tensors_of_tracer(tr, seen):
    t = tr.all_values
    key = (t.data_ptr(), t.dtype, tuple(t.shape), t.stride())
    if key not in seen:
        seen.add(key)
        yield f"tracer.{tr.name}", t


def checkpoint(sim) -> dict:
    """Snapshot of the simulation's device state (host copies) and counters."""
    torch.cuda.synchronize(sim.T.device)
    snap = {"tensors": {k: t.detach().to("cpu", copy=True) for k, t in state_tensors(sim).items()}}
    for owner, names in _HOST_COUNTERS.items():
        obj = sim if owner == "sim" else getattr(sim, owner)
        snap[owner] = {n: getattr(obj, n) for n in names if hasattr(obj, n)}
    return snap


def restore(sim, snap: dict):
    """Load a snapshot into ``sim`` (built from the same workload and
    configuration; ``start`` need not have been called)."""
    dst = state_tensors(sim)
    src = snap["tensors"]
    missing = sorted(set(src) ^ set(dst))
    if missing:
        raise ValueError(f"snapshot and simulation differ in their state fields: {missing[:8]}")
    for k, t in dst.items():
        s = src[k]
        if s.shape != t.shape or s.dtype != t.dtype:
            raise ValueError(f"field {k}: snapshot {tuple(s.shape)} {s.dtype} vs {tuple(t.shape)} {t.dtype}")
        t.copy_(s, non_blocking=False)
    for owner, vals in snap.items():
        if owner == "tensors":
            continue
        obj = sim if owner == "sim" else getattr(sim, owner)
        for n, v in vals.items():
            setattr(obj, n, v)
    torch.cuda.synchronize(sim.T.device)


def save(sim, path: str):
    snap = checkpoint(sim)
    arrays = {f"t/{k}": v.numpy() for k, v in snap["tensors"].items()}
    for owner, vals in snap.items():
        if owner == "tensors":
            continue
        for n, v in vals.items():
            arrays[f"h/{owner}/{n}"] = np.asarray(v)
    np.savez(path, **arrays)


def load(sim, path: str):
    with np.load(path) as f:
        snap = {"tensors": {}}
        for key in f.files:
            kind, rest = key.split("/", 1)
            if kind == "t":
                snap["tensors"][rest] = torch.from_numpy(f[key])
            else:
                owner, n = rest.split("/", 1)
                v = f[key]
                snap.setdefault(owner, {})[n] = v.item() if v.ndim == 0 else v
    restore(sim, snap)


# ---------------------------------------------------------------------------
# the reference's restart contract
# ---------------------------------------------------------------------------
def restart_fields(sim) -> Dict[str, Array]:
    """The fields pygetm flags ``_part_of_state`` for this configuration,
    under its names (simulation.py:572-628, momentum.py:150-164, 310-324,
    418-433, tracer.py:80, vertical_mixing.py:31-41, simulation.py:922-925)."""
    T, U, V = sim.T, sim.U, sim.V
    m = sim.momentum
    f = {"zt": T.z, "zot": T.zo, "U": m.U, "V": m.V}
    if sim.runtype > 1:
        f.update({"zint": T.zin, "ziot": T.zio, "hot": T.ho, "z0bu": U.z0b, "z0bv": V.z0b,
                  "pk": m.pk, "qk": m.qk, "Ui": m.Ui, "Vi": m.Vi, "nuh": sim.nuh, "num": sim.num})
        for tr in sim.tracers._tracers:
            f[tr.name] = tr
        if sim.delay_slow_ip:
            f.update({"SxB": m.SxB, "SyB": m.SyB})
    return f


def save_restart(sim, path: str):
    """Write the restart fields (interior and halos) to an ``.npz`` file."""
    torch.cuda.synchronize(sim.T.device)
    np.savez(path, **{n: a.all_values.detach().cpu().numpy() for n, a in restart_fields(sim).items()})


def load_restart(sim, path: str):
    """Load restart fields before ``start`` (simulation.py:128-202): every
    field of the state must be present."""
    fields = restart_fields(sim)
    with np.load(path) as f:
        missing = [n for n in fields if n not in f.files]
        if missing:
            raise Exception("The following field(s) are part of the model state but not found "
                            f"in {path!r}: {', '.join(missing)}")
        for n, a in fields.items():
            a.all_values.copy_(torch.from_numpy(f[n]))
