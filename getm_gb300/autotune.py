"""Launch-shape autotuner for the hot kernels.

The library reads five launch-shape knobs at every launch (``getm_tune_set``,
per host thread): the rows per block of the x advection pass, the rows a warp
marches in the 3D y pass, the rows of 32 columns per block of the column
kernels (w pass, float column solve), the blocks per SM of the one-launch
2D substep and the form of the 3D x pass (four cells or one cell per lane).  The best shapes depend on the domain: a 64 x 64 x 20 member has
too few columns to fill 152 SMs with 8-row blocks, a 400 x 300 x 40 box has
plenty.

``search`` is a coordinate descent over the knobs with any timing function
(a step of a real simulation on the GPU in ``tune``; a model in the tests).
Results are kept per size bucket (precision, horizontal points in
half-octaves, layers in tens) in a JSON file; ``lookup`` returns the shapes
of the nearest tuned bucket.  A CUDA graph keeps the shapes it was captured
with, so applying a domain's shapes before capturing its step gives every
member of an ensemble its own shapes.
"""

from __future__ import annotations

import json
import math
import threading
from pathlib import Path
from typing import Callable, Dict, Iterable, Optional, Tuple

# name -> (knob index of include/getm_gb300.h, candidate values); the first
# candidate listed for each knob is not necessarily the default
KNOBS: Dict[str, Tuple[int, Tuple[int, ...]]] = {
    "xpass_rows": (0, (2, 4, 8)),
    "ymarch_chunk": (1, (16, 32, 64)),
    "column_rows": (2, (1, 2, 4)),
    "substep_blocks_per_sm": (3, (0, 1)),
    "xpass_vec": (4, (1, 0)),
    "column_solve": (5, (0, 1)),
}
DEFAULTS: Dict[str, int] = {"xpass_rows": 8, "ymarch_chunk": 32, "column_rows": 4, "substep_blocks_per_sm": 0,
                            "xpass_vec": 1, "column_solve": 0}
# knobs of kernels that only the mixed form runs
FLOAT_ONLY = frozenset({"column_solve"})
CACHE_PATH = Path(__file__).resolve().parent / "tiles.json"

_applied = threading.local()


def apply(tiles: Optional[Dict[str, int]]) -> None:
    """Set the calling thread's knobs (missing names keep their defaults);
    nothing is called when they are already set."""
    want = dict(DEFAULTS)
    if tiles:
        for k, v in tiles.items():
            if k not in KNOBS:
                raise KeyError(f"unknown launch-shape knob {k!r}")
            want[k] = int(v)
    if getattr(_applied, "tiles", None) == want:
        return
    from ._lib import call

    for k, v in want.items():
        call("getm_tune_set", KNOBS[k][0], v)
    _applied.tiles = want


def current() -> Dict[str, int]:
    """The calling thread's knob values, read back from the library."""
    import ctypes

    from ._lib import call

    out = {}
    for k, (idx, _) in KNOBS.items():
        v = ctypes.c_int(0)
        call("getm_tune_get", idx, ctypes.addressof(v))
        out[k] = v.value
    return out


def bucket(nx: int, ny: int, nz: int, precision: str) -> str:
    """Size bucket of a domain: precision, horizontal points in half-octaves
    (log2 rounded to 0.5) and layers rounded to tens."""
    hp = round(2.0 * math.log2(max(nx * ny, 1))) / 2.0
    return f"{precision}/p{hp:g}/z{int(round(nz / 10.0)) * 10}"


def _parse(key: str) -> Tuple[str, float, int]:
    prec, p, z = key.split("/")
    return prec, float(p[1:]), int(z[1:])


def search(measure: Callable[[Dict[str, int]], float], knobs: Dict[str, Tuple[int, Tuple[int, ...]]] = KNOBS,
           start: Optional[Dict[str, int]] = None, rounds: int = 2) -> Tuple[Dict[str, int], float, list]:
    """Coordinate descent: starting from ``start`` (default: DEFAULTS), try
    every candidate of one knob with the others fixed, keep the fastest, go
    on to the next knob; repeat ``rounds`` times or until nothing changes.
    ``measure(tiles)`` returns the time of one step with those shapes.
    Returns (best shapes, best time, [(shapes, time), ...] of every trial)."""
    best = dict(start or DEFAULTS)
    trials = []
    seen: Dict[Tuple, float] = {}

    def timed(t):
        key = tuple(sorted(t.items()))
        if key not in seen:
            seen[key] = float(measure(dict(t)))
            trials.append((dict(t), seen[key]))
        return seen[key]

    best_t = timed(best)
    for _ in range(max(1, rounds)):
        changed = False
        for name, (_, cands) in knobs.items():
            for v in cands:
                if v == best[name]:
                    continue
                t = dict(best, **{name: v})
                tt = timed(t)
                if tt < best_t:
                    best, best_t, changed = t, tt, True
        if not changed:
            break
    return best, best_t, trials


class TileCache:
    """Tuned shapes per size bucket, kept in a JSON file."""

    def __init__(self, entries: Optional[dict] = None):
        self.entries: Dict[str, dict] = dict(entries or {})

    @classmethod
    def load(cls, path=CACHE_PATH) -> "TileCache":
        p = Path(path)
        return cls(json.loads(p.read_text())["buckets"] if p.exists() else {})

    def save(self, path=CACHE_PATH) -> None:
        Path(path).write_text(json.dumps({"buckets": dict(sorted(self.entries.items()))}, indent=1) + "\n")

    def store(self, nx, ny, nz, precision, tiles, ms, default_ms, domain: str = "") -> None:
        self.entries[bucket(nx, ny, nz, precision)] = {"tiles": dict(tiles), "ms_per_step": ms,
                                                       "default_ms_per_step": default_ms, "domain": domain}

    def lookup(self, nx: int, ny: int, nz: int, precision: str) -> Dict[str, int]:
        """Shapes of the exact bucket, else of the nearest bucket of the same
        precision (distance in half-octaves of points plus tens of layers),
        else the defaults."""
        key = bucket(nx, ny, nz, precision)
        if key in self.entries:
            return dict(self.entries[key]["tiles"])
        _, hp, z = _parse(key)
        best, dist = None, None
        for k, e in self.entries.items():
            pr, hp2, z2 = _parse(k)
            if pr != precision:
                continue
            d = abs(hp2 - hp) * 2.0 + abs(z2 - z) / 10.0
            if dist is None or d < dist:
                best, dist = e, d
        return dict(best["tiles"]) if best is not None else dict(DEFAULTS)


def lookup(nx: int, ny: int, nz: int, precision: str, path=CACHE_PATH) -> Dict[str, int]:
    """Tuned shapes for a domain from the committed cache."""
    return TileCache.load(path).lookup(nx, ny, nz, precision)


# ---------------------------------------------------------------------------
# measurement on the GPU
# ---------------------------------------------------------------------------
def step_timer(sim, replays: int = 4) -> Callable[[Dict[str, int]], float]:
    """A ``measure`` function for ``search``: with the given shapes applied,
    capture two 3D steps of ``sim`` (both u/v orders) into CUDA graphs and
    time ``replays`` replays of each with CUDA events; returns ms per 3D
    step.  The simulation keeps advancing (use a scratch copy)."""
    import torch

    def measure(tiles: Dict[str, int]) -> float:
        apply(tiles)
        dev = sim.T.device
        stream = torch.cuda.Stream(device=dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        graphs = []
        with torch.cuda.stream(stream):
            for _ in range(2):
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=stream):
                    for _ in range(sim.split_factor):
                        sim.advance()
                graphs.append(g)
        torch.cuda.current_stream(dev).wait_stream(stream)
        for g in graphs:
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(replays):
            for g in graphs:
                g.replay()
        e1.record()
        torch.cuda.synchronize(dev)
        if sim.split2d_status() != 0:
            raise RuntimeError("one-launch substep reported an error while tuning")
        del graphs
        return e0.elapsed_time(e1) / (2 * replays)

    return measure


def tune(sim, rounds: int = 2, replays: int = 4, only: Optional[Iterable[str]] = None,
         start: Optional[Dict[str, int]] = None) -> Tuple[Dict[str, int], float, float, list]:
    """Tune the shapes on a started simulation (warmed up here with two eager
    3D steps).  ``only``: search just these knobs; ``start``: the shapes to
    start from (default: DEFAULTS), e.g. a bucket's cached shapes when a knob
    is added.  Returns (shapes, ms per step, ms per step with the starting
    shapes, trials).  Leaves the defaults applied."""
    import torch

    apply(None)
    for _ in range(2 * sim.split_factor):
        sim.advance()
    torch.cuda.synchronize(sim.T.device)
    measure = step_timer(sim, replays)
    knobs = {k: v for k, v in KNOBS.items() if only is None or k in set(only)}
    if sim._split2d is None:  # no one-launch substep in this configuration
        knobs.pop("substep_blocks_per_sm", None)
    if sim.precision != "mixed":
        for k in FLOAT_ONLY:
            knobs.pop(k, None)
    first = dict(DEFAULTS, **(start or {}))
    best, t, trials = search(measure, knobs=knobs, start=first, rounds=rounds)
    first_t = next(tt for tl, tt in trials if tl == first)
    apply(None)
    return best, t, first_t, trials


def _applies(precision: str, only: Optional[Iterable[str]]) -> bool:
    """Whether a search over the knobs ``only`` (None: all) has anything to
    tune in a domain of this precision."""
    return only is None or precision == "mixed" or any(k not in FLOAT_ONLY for k in only)


def _tune_main(argv: Optional[Iterable[str]] = None) -> None:
    """Tune the benchmark domains and a ladder of ensemble-member sizes and
    write the cache (run on the GPU)."""
    import argparse

    import numpy as np
    import torch

    from . import workloads
    from .ensemble import make_member
    from .simulation import Simulation

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(CACHE_PATH))
    ap.add_argument("--sides", default="64,96,128,192,256,384,512")
    ap.add_argument("--nzs", default="20,30,40")
    ap.add_argument("--no-seamount", action="store_true")
    ap.add_argument("--knobs", default="", help="search only these knobs (comma-separated)")
    ap.add_argument("--refine", action="store_true",
                    help="start each bucket from its cached shapes (and keep its reference time)")
    args = ap.parse_args(list(argv) if argv is not None else None)
    cache = TileCache.load(args.out)
    only = [k for k in args.knobs.split(",") if k] or None
    for k in only or ():
        if k not in KNOBS:
            raise SystemExit(f"unknown knob {k!r}")

    def run(sim, nx, ny, nz, prec, domain, replays):
        key = bucket(nx, ny, nz, prec)
        old = cache.entries.get(key) if args.refine else None
        best, t, t0, _ = tune(sim, replays=replays, only=only, start=old["tiles"] if old else None)
        # the time with the defaults stays the one measured in the full search
        default_t = old["default_ms_per_step"] if old else t0
        cache.store(nx, ny, nz, prec, best, t, default_t, domain)
        return best, t, t0

    dev = "cuda"
    sides = [int(s) for s in args.sides.split(",") if s]
    nzs = [int(s) for s in args.nzs.split(",") if s]
    rng = np.random.default_rng(11)
    for n in sides:
        for nz in nzs:
            wl = workloads.ensemble_member(rng, nmin=n, nmax=n, nzmin=nz, nzmax=nz)
            sim = make_member(wl, "mixed", device=dev)
            best, t, t0 = run(sim, wl.T.nx, wl.T.ny, wl.T.nz, "mixed", "ensemble member", 4)
            print(f"member {wl.T.nx}x{wl.T.ny}x{wl.T.nz}: {best} {t:.3f} ms/step (start {t0:.3f})", flush=True)
            del sim
            torch.cuda.empty_cache()
    # the benchmark domains last: a member of the same size bucket must not
    # overwrite their shapes
    if not args.no_seamount:
        wl = workloads.seamount()
        p = wl.params
        for prec in [p for p in ("mixed", "fp64") if _applies(p, only)]:
            sim = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=prec, device=dev)
            zc = sim.T.zc.all_values
            sim.temp.all_values.copy_(torch.where(sim.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                                                  sim.temp.all_values.double()))
            sim.start(p["timestep"], p["split_factor"])
            best, t, t0 = run(sim, wl.T.nx, wl.T.ny, wl.T.nz, prec, "seamount", 3 if prec == "fp64" else 6)
            print(f"seamount {prec}: {best} {t:.3f} ms/step (start {t0:.3f})", flush=True)
            del sim
            torch.cuda.empty_cache()
    cache.save(args.out)


if __name__ == "__main__":
    _tune_main()
