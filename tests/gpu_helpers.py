"""Helpers for GPU parity tests: one HostGrid, an oracle copy and a device
copy with identical random time-varying fields."""

from __future__ import annotations

import numpy as np

from getm_gb300.domain import FILL_VALUE


def random_state(Th, rng, nz):
    """Random positive D/hn/ho on every grid of the tree (masked points keep
    FILL_VALUE as in pygetm), as numpy dicts keyed by grid postfix."""
    state = {}
    for g in Th.all_grids():
        water = g.mask != 0
        D = np.where(water, g.H * rng.uniform(0.9, 1.1, g.H.shape), FILL_VALUE)
        frac = rng.uniform(0.5, 1.5, (nz,) + D.shape)
        frac /= frac.sum(axis=0, keepdims=True)
        hn = np.where(water[None], frac * D[None], FILL_VALUE)
        ho = np.where(water[None], hn * rng.uniform(0.95, 1.05, hn.shape), FILL_VALUE)
        state[g.postfix] = dict(D=D, hn=hn, ho=ho)
    return state


def apply_state_oracle(Tor, state):
    import oracle.oracle as O  # noqa: F401

    def walk(g, seen):
        if g is None or id(g) in seen:
            return
        seen.add(id(g))
        s = state[g.postfix]
        g.D[...] = s["D"]
        g.hn[...] = s["hn"]
        g.ho[...] = s["ho"]
        for c in (g.ugrid, g.vgrid, g.xgrid):
            walk(c, seen)

    walk(Tor, set())


def apply_state_device(Tdev, state):
    import torch

    from getm_gb300.core import CENTERS, Array

    for g in Tdev.all_grids():
        s = state[g.postfix]
        g.D.all_values.copy_(torch.from_numpy(s["D"]))
        g.hn.all_values.copy_(torch.from_numpy(s["hn"]))
        g.ho = Array(g, torch.from_numpy(s["ho"]).to(g.device), z=CENTERS, name="ho" + g.postfix)


def dev(a, device="cuda"):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def host(t):
    return t.detach().cpu().numpy()


def oracle_variant(variant: str):
    """Context manager: every oracle call inside runs the given build of the
    C restatement ("serial": no contraction; "fma": multiply-adds contracted
    as gfortran does on aarch64)."""
    import contextlib

    import oracle.oracle as O

    @contextlib.contextmanager
    def cm():
        old = O._lib
        O._lib = O.load_variant(variant)
        try:
            yield
        finally:
            O._lib = old

    return cm()


def relative_errors(a: dict, b: dict) -> dict:
    """max |a - b| / max |b| per field over each field's water points; a and
    b map names to (array, mask) or (array, mask, scale) with the same keys."""
    out = {}
    for k, v in b.items():
        x, m = v[0], v[1]
        y = a[k][0]
        wet = np.broadcast_to(m, x.shape)
        xs, ys = x[wet], y[wet]
        # an optional third entry: the scale to measure against (for a field
        # that is the small difference of two larger terms)
        scale = v[2] if len(v) > 2 else (np.abs(xs).max() if xs.size else 0.0)
        out[k] = float(np.abs(ys - xs).max() / scale) if scale > 0 else float(np.abs(ys - xs).max(initial=0.0))
    return out
