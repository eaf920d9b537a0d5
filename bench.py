"""Benchmark: 3D cell-updates/s of the split-explicit baroclinic step.

Workload: the seamount box of 400 x 300 x 40 sigma layers (dx = 2 km, 4500 m
deep, 4000 m Gaussian seamount, linear stratification, nonlinear EOS,
Shchepetkin-McWilliams internal pressure, dt2d = 4 s, 30 substeps per 3D step,
f = 1e-4, log-law bottom drag).  One step = one 3D (macro) time step with its
30 2D substeps and both active tracers.  Unit of work: one cell-update = one
interior T cell (land included) advanced by one 3D step.

Our arm (default): the mixed-precision GPU path (``--precision fp64`` for the
plain form; the other form is measured beside it, with the mixed form's error
against FP64), state resident in HBM, the two-3D-step sequence replayed from
a CUDA graph, timed with CUDA events.  ``e2e`` repeats
the timing through the public API with the per-step surface forcing copied
host->device from pinned memory and the surface elevation copied back.
``--impl reference``: the reference's CPU algorithm (the C/numpy oracle
restatement, OpenMP over all host cores) on a bounded sample of the same
workload.  Multi-GPU: independent replicas (one domain per GPU, no
collective); the value is the sum over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# CUDA settings read when the process creates its context (before torch
# touches the GPU): every kernel loaded with the context instead of at its
# first launch (a first launch on a busy device holds up the other threads'
# CUDA calls: the serving loop's step issue while a request is set up), and
# 32 hardware work queues, one per lane stream of the serving and ensemble
# legs (with the default 8, lanes that share a queue wait on each other).
os.environ.setdefault("CUDA_MODULE_LOADING", "EAGER")
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--tracer-storage", choices=["float64", "float32"], default=None,
                    help="tracer type of the mixed form (default float64)")
    ap.add_argument("--no-compare", action="store_true", help="skip the other precision form")
    ap.add_argument("--nx", type=int, default=400)
    ap.add_argument("--ny", type=int, default=300)
    ap.add_argument("--nz", type=int, default=40)
    ap.add_argument("--error-steps", type=int, default=1000,
                    help="3D steps after which the mixed form is compared with FP64 (0: skip)")
    ap.add_argument("--ensemble", type=int, default=256, help="members of the batched ensemble (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=8)
    ap.add_argument("--serve-rates", default="50,100,200,400",
                    help="Poisson request rates, 1/s, comma-separated ('' : skip)")
    ap.add_argument("--serve-duration", type=float, default=5.0, help="seconds of arrivals per rate and form")
    ap.add_argument("--no-c1", dest="c1", action="store_false",
                    help="skip the 120x100x30 tracer-transport leg")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--shelf-steps", type=int, default=100,
                    help="3D steps of the 20-tracer shelf sea, both forms, for its error report (0: skip)")
    ap.add_argument("--shelf-size", default="1000x800x30")
    ap.add_argument("--no-column-solve", dest="column_solve", action="store_false",
                    help="skip timing the two float column solves")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(x: float, device) -> float:
    """The largest of every rank's x (one process per GPU, each with its own
    replica of the domain); a single process returns x."""
    ws, _, _ = _dist()
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _whole_job_rate(cells: int, nsteps: int, ms: float) -> float:
    """Cell-updates per second of the whole job: every rank advances its own
    replica of `cells` cells by nsteps 3D steps, and the job takes the slowest
    rank's time `ms` (milliseconds)."""
    ws, _, _ = _dist()
    return cells * nsteps * ws / (ms / 1000.0)


def _host_threads() -> int:
    """Threads of the CPU legs: OMP_NUM_THREADS where set, else every core."""
    try:
        return max(1, int(os.environ["OMP_NUM_THREADS"]))
    except (KeyError, ValueError):
        return os.cpu_count() or 1


def cpu_reference(args, nmacro: int, threads: int):
    """Time the oracle restatement of the reference's CPU path."""
    import numpy as np

    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    os.environ.setdefault("GETM_ORACLE_VARIANT", "omp" if threads > 1 else "serial")
    from getm_gb300 import workloads
    from oracle import models

    wl = workloads.seamount(nx=args.nx, ny=args.ny, nz=args.nz)
    p = wl.params
    s = models.Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    s.temp[...] = np.where(s.T.mask[None] != 0, workloads.seamount_temperature(s.T.zc), s.temp)
    s.start(p["timestep"], p["split_factor"])
    t0 = time.perf_counter()
    for _ in range(nmacro * p["split_factor"]):
        s.advance()
    dt = time.perf_counter() - t0
    return wl.cells * nmacro / dt, dt


def _config(wl, ws):
    """The workload's description, identical in both arms."""
    return {"workload": f"seamount {wl.T.nx}x{wl.T.ny}x{wl.T.nz} baroclinic split-explicit, "
                        f"{wl.params['split_factor']} substeps per 3D step",
            "cells": wl.cells, "wet_cells": wl.wet_cells,
            "l2": "working set (> 1 GB of 3D fields) exceeds L2; no flush needed",
            "parallelism": f"replicas x{ws}"}


REFERENCE_BUDGET_S = 240.0  # timed CPU work of the reference arm


def run_reference(args):
    """The reference's CPU algorithm (the oracle restatement, OpenMP on every
    host core) on the same workload: W warm-up 3D steps (at most 2: the CPU
    has nothing to warm), then K timed 3D steps, stopping early only if the
    timed work would exceed a few minutes (the line then says how many ran)."""
    import numpy as np

    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = _host_threads()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    os.environ.setdefault("GETM_ORACLE_VARIANT", "omp" if threads > 1 else "serial")
    from getm_gb300 import workloads
    from oracle import models

    wl = workloads.seamount(nx=args.nx, ny=args.ny, nz=args.nz)
    p = wl.params
    s = models.Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"])
    s.temp[...] = np.where(s.T.mask[None] != 0, workloads.seamount_temperature(s.T.zc), s.temp)
    s.start(p["timestep"], p["split_factor"])
    nwarm = min(args.warmup, 2)
    for _ in range(nwarm * p["split_factor"]):
        s.advance()
    done, t0 = 0, time.perf_counter()
    while done < args.steps:
        for _ in range(p["split_factor"]):
            s.advance()
        done += 1
        el = time.perf_counter() - t0
        if el * (done + 1) / done > REFERENCE_BUDGET_S:
            break
    dt = time.perf_counter() - t0
    value = wl.cells * done / dt
    sample = f"{done} of {args.steps} 3D steps timed" if done < args.steps else f"{done} 3D steps"
    line = {"metric": "3D cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": done, "warmup": nwarm, "ms_per_step": 1000.0 * dt / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": _config(wl, ws), "impl": "reference", "form": "fp64 (CPU restatement, OpenMP)",
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample + " of the full workload"},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _make_sim(wl, precision, device, round_to_float32=True, tracer_storage=None, ip_arithmetic=None):
    """Seamount simulation from rest; the initial temperature (20 -> 4 degC,
    linear in depth) is rounded to float32 unless told otherwise, so both
    forms start from identical fields.  ``tracer_storage``: the mixed form's
    tracer type (default float64); ``ip_arithmetic``: its internal-pressure
    arithmetic (default float32 slope corrections)."""
    import torch

    from getm_gb300.simulation import Simulation

    p = wl.params
    sim = Simulation(wl.T, wl.dga, num=p["num"], nuh=p["nuh"], precision=precision, device=device, tiles="auto",
                     tracer_storage=tracer_storage, internal_pressure_arithmetic=ip_arithmetic)
    zc = sim.T.zc.all_values
    temp0 = torch.where(sim.T.mask.all_values[None] != 0, 4.0 + 16.0 * (zc + 4500.0) / 4500.0,
                        sim.temp.all_values.double())
    if round_to_float32:
        temp0 = temp0.float().double()
    sim.temp.all_values.copy_(temp0)
    sim.start(p["timestep"], p["split_factor"])
    return sim


class Runner:
    """Warm-up, CUDA-graph capture and replay of one simulation: one graph
    per 3D step parity (the 3D momentum update alternates its u/v order each
    step), so every replay is exactly one 3D step with its substeps."""

    period = 2

    def __init__(self, sim, warmup, use_graph, hook=None):
        import torch

        from getm_gb300 import _lib

        self.sim = sim
        self.hook = hook
        self.totals0 = sim.totals_device().clone()
        nwarm = max(warmup, 3)
        nwarm += nwarm % self.period  # captured steps start on an even 3D step
        for _ in range(nwarm):
            self._step3d()
        self.steps_done = nwarm  # 3D steps run on the device so far
        torch.cuda.synchronize()
        n0 = _lib.launch_count()
        self.graphs = None
        if use_graph:
            stream = torch.cuda.Stream()
            stream.wait_stream(torch.cuda.current_stream())
            self.graphs = []
            with torch.cuda.stream(stream):
                for _ in range(self.period):
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=stream):
                        self._step3d()
                    self.graphs.append(g)
            torch.cuda.current_stream().wait_stream(stream)
            self.launches_per_period = _lib.launch_count() - n0
            for g in self.graphs:  # capture runs nothing: one untimed replay of each
                g.replay()
            self.steps_done += self.period
        else:
            for _ in range(self.period):
                self._step3d()
            self.launches_per_period = _lib.launch_count() - n0
            self.steps_done += self.period
        torch.cuda.synchronize()
        self.check()

    def _step3d(self):
        for _ in range(self.sim.split_factor):
            self.sim.advance()
        if self.hook is not None:
            self.hook(self.sim)

    def check(self):
        """Raise if a grid barrier of the one-launch substep gave up (its
        substeps would then have done no work)."""
        st = self.sim.split2d_status()
        if st != 0:
            raise RuntimeError(f"one-launch substep reported status {st}: a grid barrier gave up")

    def run_step(self):
        """One 3D step (graph replay of the step's parity)."""
        if self.graphs is not None:
            self.graphs[self.steps_done % self.period].replay()
        else:
            self._step3d()
        self.steps_done += 1

    def run_period(self):
        for _ in range(self.period):
            self.run_step()

    def run_to(self, nsteps):
        while self.steps_done < nsteps:
            self.run_step()

    def timed(self, nsteps, clocks_index=None):
        import torch

        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        sampler = ClockSampler(clocks_index) if clocks_index is not None else None
        if sampler:
            sampler.__enter__()
        start.record()
        for _ in range(nsteps):
            self.run_step()
        end.record()
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__(None, None, None)
        self.check()
        return start.elapsed_time(end), (sampler.summary() if sampler else None)


# dram__bytes_read.sum + dram__bytes_write.sum of one launch on the
# 400 x 300 x 40 seamount, from ncu captures of this bench (profiles/); None:
# not captured.  The x pass over both tracers, by (storage suffix, four
# cells per lane): profiles/hpass_x_f64s_seamount_400x300x40.md (184.0 +
# 83.0 MB), and the float-storage one-cell pass of an earlier capture.
TRAFFIC_X_PASS = {("_f32", 0): 152.51e6, ("_f64s", 1): 267.0e6, ("_f64s", 0): 263.9e6}
# one one-launch substep, by form: profiles/substep_2d_seamount_400x300.md
# (60.8 + 5.3 MB; the plane's fields stay in L2)
TRAFFIC_SUBSTEP = {"mixed": 66.1e6}


def _roofline(sim, peak, peak_kind):
    """Time the dominant kernel alone on the live state: one x-direction
    advection pass of both tracers (hpass_x_kernel, one launch)."""
    import torch

    from getm_gb300 import _lib

    T = sim.T
    tr = sim.tracers
    adv = tr._advection
    u = sim.momentum.uk.all_values
    hu = T.ugrid.hn.all_values
    h_in = T.hn.all_values
    h_out = torch.empty_like(h_in)
    fin = [x.all_values for x in tr._tracers]
    fout = [torch.empty_like(x) for x in fin]
    from getm_gb300.core import _sfx_storage

    sfx = _sfx_storage([u], fin)
    pin = _lib.ptr_array([x.data_ptr() for x in fin])
    pout = _lib.ptr_array([x.data_ptr() for x in fout])
    stream = torch.cuda.current_stream().cuda_stream

    def launch():
        _lib.call("getm_advection_uv_pass" + sfx, 1, T.nz, adv.p, T.handle, T.ugrid.handle, u.data_ptr(), None,
                  0.5 * sim.macrotimestep, h_in.data_ptr(), h_out.data_ptr(), hu.data_ptr(), len(fin), pin, pout,
                  stream)

    launch()
    torch.cuda.synchronize()
    reps = 50
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(reps):
        launch()
    ev1.record()
    torch.cuda.synchronize()
    t_kernel = ev0.elapsed_time(ev1) / reps / 1000.0
    # interior cells of the layers the pass updates (halos excluded)
    n3 = T.nx * T.ny * T.nz
    sz = u.element_size()
    fsz = fin[0].element_size()
    # u, hu, h in + h out + per tracer in + out (each 3D field read or written once)
    alg = n3 * (sz + 8 + 8 + 8 + len(fin) * 2 * fsz)
    achieved = alg / t_kernel / 1e9
    # the four-cells-per-lane form runs where the knob asks for it and rows
    # are whole 16-byte vectors
    from getm_gb300 import autotune

    vec = int(sfx != "" and autotune.current()["xpass_vec"] == 1 and T.nx_ % 4 == 0)
    kernel = {("_f32", 0): "hpass_x_inc_kernel<float, float>", ("_f32", 1): "hpass_x_vec_kernel<float, float>",
              ("_f64s", 0): "hpass_x_inc_kernel<double, float>", ("_f64s", 1): "hpass_x_vec_kernel<double, float>",
              ("", 0): "hpass_x_kernel<double>"}[(sfx, vec)]
    # DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
    # of this kernel on this workload, from an ncu capture of this bench
    traffic = TRAFFIC_X_PASS.get((sfx, vec))
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": f"{kernel} (2 tracers)",
            "bytes_per_launch": alg, "us_per_launch": t_kernel * 1e6, "peak_kind": peak_kind}


def _column_solve_leg(sim, device):
    """The mixed form's float column solve of both FP64-stored tracers (one
    getm_vertical_diffusion_batch_f64s call) timed with CUDA events, one
    thread per column against the segmented solve (GETM_TUNE_COLUMN_SOLVE),
    on copies of the live seamount tracers and on small seamounts of
    ensemble-member size."""
    import torch

    from getm_gb300 import autotune, workloads
    from getm_gb300.core import Array, CENTERS

    def time_solves(s):
        T = s.T
        vd = s.tracers._vertical_diffusion
        fields = [Array(T, t.all_values.clone(), z=CENTERS) for t in s.tracers._tracers]
        mol = [t.molecular_diffusivity for t in s.tracers._tracers]
        n3 = T.nx * T.ny * T.nz
        out = {"domain": f"{T.nx}x{T.ny}x{T.nz}"}
        for name, knob in (("thread_per_column", 0), ("segmented", 1)):
            autotune.apply(dict(s.tiles or {}, column_solve=knob))
            for _ in range(3):
                vd.batch(s.nuh, s.macrotimestep, fields, mol, None, [None] * len(fields))
            torch.cuda.synchronize()
            reps = 20
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                vd.batch(s.nuh, s.macrotimestep, fields, mol, None, [None] * len(fields))
            e1.record()
            torch.cuda.synchronize()
            us = e0.elapsed_time(e1) / reps * 1000.0
            # nuh (float) and both thicknesses read, two FP64 fields read and written
            alg = n3 * (4 + 8 + 8 + len(fields) * 16)
            out[name] = {"us": us, "gbs": alg / us / 1e3}
        autotune.apply(s.tiles)
        out["speedup"] = out["thread_per_column"]["us"] / out["segmented"]["us"]
        return out

    res = [time_solves(sim)]
    for nx, ny, nz in ((64, 64, 20), (128, 128, 30), (256, 192, 40)):
        s = _make_sim(workloads.seamount(nx=nx, ny=ny, nz=nz, dx=2000.0 * 400 / nx), "mixed", device)
        s.advance()
        res.append(time_solves(s))
        del s
    return res


def _round_tracers(sim):
    for tr in (sim.temp, sim.salt):
        tr.all_values.copy_(tr.all_values.float().double())


def _errors(wl, runners, args, device):
    """Advance both forms to the same 3D step and compare fields and
    compensated domain totals.  A third run, FP64 arithmetic whose tracers are
    rounded to float32 after every 3D step, shows the error that float32
    storage of the tracers alone causes (the floor for any form that stores
    them in float32).  A fourth, the mixed form with its internal pressure
    gradient evaluated in FP64, shows how much of the flow's error the float
    slope corrections cause, and what removing it costs per 3D step."""
    import torch

    target = max(args.error_steps, max(r.steps_done for r in runners.values()))
    cond = Runner(_make_sim(wl, "fp64", device), args.warmup, not args.no_graph, hook=_round_tracers)
    ip64 = Runner(_make_sim(wl, "mixed", device, ip_arithmetic="float64"), args.warmup, not args.no_graph)
    for r in list(runners.values()) + [cond]:
        r.run_to(target)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = ip64.steps_done
    e0.record()
    ip64.run_to(target)
    e1.record()
    torch.cuda.synchronize()
    ip64_ms = e0.elapsed_time(e1) / max(target - n0, 1)
    ip64.check()
    steps = {r.steps_done for r in list(runners.values()) + [cond, ip64]}
    assert len(steps) == 1, steps
    wet = torch.from_numpy(wl.T.mask == 1).to(device)
    uwet = torch.from_numpy(wl.T.ugrid.mask == 1).to(device)

    def rel(x, y, m=wet):
        x = x.double()[..., m]
        y = y.double()[..., m]
        return float((x - y).abs().max() / y.abs().max())

    def compare(a, b):
        # z: max error over the FP64 run's range of z (the seamount's z is a
        # residual of a few micrometres: the tidal shelf sea gives the
        # meaningful elevation figure); z_abs_m in metres
        za, zb = a.T.z.all_values[wet], b.T.z.all_values[wet]
        return {"temp": rel(a.temp.all_values, b.temp.all_values), "salt": rel(a.salt.all_values, b.salt.all_values),
                "z": float((za - zb).abs().max() / (zb.max() - zb.min())), "z_abs_m": float((za - zb).abs().max()),
                "z_max_m": float(zb.abs().max()), "U": rel(a.momentum.U.all_values, b.momentum.U.all_values, uwet),
                "uk": rel(a.momentum.uk.all_values, b.momentum.uk.all_values, uwet)}

    a, b = runners["mixed"], runners["fp64"]
    out = {"steps": steps.pop()}
    out.update(compare(a.sim, b.sim))
    ta, tb = a.sim.totals_device(), b.sim.totals_device()
    names = ["volume", "temp", "salt"]
    out["totals_vs_fp64"] = {n: float((x - y) / y) for n, x, y in zip(names, ta.tolist(), tb.tolist())}
    out["totals_drift"] = {f: {n: float((x - y) / y) for n, x, y in
                               zip(names, r.sim.totals_device().tolist(), r.totals0.tolist())}
                           for f, r in (("mixed", a), ("fp64", b))}
    out["fp64_with_float32_tracer_storage"] = compare(cond.sim, b.sim)
    out["mixed_with_fp64_internal_pressure"] = dict(compare(ip64.sim, b.sim), ms_per_step=ip64_ms)
    return out


def _pcts(deltas):
    import numpy as np

    d = np.asarray([x for x in deltas if x > 0.0])
    if not d.size:
        return None, None
    return float(np.percentile(d, 50) * 1e3), float(np.percentile(d, 99) * 1e3)


def _ensemble_leg(args, device):
    """Batched ensemble of independent domains (mixed form, each member with
    the tuned launch shapes of its size), two ways on the same members:
    (a) every member's 3D step is one graph replay on one of 16 lane
    streams; (b) the 2D substeps of all members run as one persistent
    cooperative launch per substep index, then every member's 3D step on the
    lanes.  Throughput of both against the members replayed one after
    another, and the per-member step latency.  Set-up happens before the
    timed regions."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.ensemble import BatchedEnsemble, Ensemble, make_member

    wls = workloads.ensemble(args.ensemble, seed=4)
    main = torch.cuda.current_stream()
    steps = max(args.ensemble_steps, 2)

    def timed(step, n, nsteps):
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n)] for _ in range(nsteps)]
        torch.cuda.synchronize()
        start.record(main)
        for q in range(nsteps):
            step(evs[q])
        end.record(main)
        torch.cuda.synchronize()
        deltas = []
        for m in range(n):
            times = [start.elapsed_time(evs[q][m]) / 1000.0 for q in range(nsteps)]
            deltas += [b - a for a, b in zip(times, times[1:])]
        return start.elapsed_time(end) / 1000.0, deltas

    t_setup = time.perf_counter()
    ens = Ensemble([make_member(w, "mixed", device, tiles="auto") for w in wls], lanes=16)
    ens.prepare()
    t_setup = time.perf_counter() - t_setup
    n = len(ens.runners)
    cells = ens.cells
    ens.step()  # one untimed replay of every graph
    t_conc, d_conc = timed(lambda e: ens.step(events=e), n, steps)
    t_seq, _ = timed(lambda e: ens.step(sequential=True, events=e), n, 2)
    conc, seq = cells * steps / t_conc, cells * 2 / t_seq
    p50, p99 = _pcts(d_conc)
    del ens
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    t_bsetup = time.perf_counter()
    bat = BatchedEnsemble([make_member(w, "mixed", device, substep_kernel=True, tiles="auto") for w in wls],
                          lanes=16)
    bat.prepare()
    t_bsetup = time.perf_counter() - t_bsetup
    bat.step()
    t_bat, d_bat = timed(lambda e: bat.step(events=e), n, steps)
    torch.cuda.synchronize()
    if bat.status() != 0:
        raise RuntimeError("batched substep reported a barrier error")
    bp50, bp99 = _pcts(d_bat)
    out = {"members": n, "cells": cells, "lanes": 16, "steps": steps, "unit": "cell-updates/s",
           "precision": "mixed", "tiles": "tuned per member size (autotune cache)",
           "workload": "256-type ensemble: sides log-uniform 64-256, nz 20-40, 20-40 substeps, seed 4",
           "value": max(conc, cells * steps / t_bat),
           "lane_graphs": {"value": conc, "member_step_latency_p50_ms": p50, "member_step_latency_p99_ms": p99,
                           "setup_s": t_setup},
           "batched_substeps": {"value": cells * steps / t_bat, "member_step_latency_p50_ms": bp50,
                                "member_step_latency_p99_ms": bp99, "setup_s": t_bsetup,
                                "launches_per_round": max(bat.nsub) + n},
           "sequential_value": seq}
    out["speedup_vs_sequential"] = out["value"] / seq
    del bat
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def _serving_leg(args, device):
    """Continuous batching of Poisson request streams at each rate (both
    forms, one after the other, the same requests): per-step latency
    p50/p99, admitted and finished requests and throughput."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.serving import GB, Server, summarize

    rates = [float(x) for x in args.serve_rates.split(",") if x.strip()]
    out = {"arrival_window_s": args.serve_duration, "deadline_s": 3.0 * args.serve_duration,
           "budget_gb": args.serve_budget_gb, "lanes": 32,
           "requests": "sides log-uniform 64-512, nz 20-40, 10-200 3D steps, seed 5", "rates": {}}
    for rate in rates:
        per = {}
        for prec in ("mixed", "fp64"):
            reqs = workloads.serving_requests(rate, args.serve_duration, seed=5, precision=prec)
            srv = Server(budget_bytes=args.serve_budget_gb * GB, lanes=32, device=device)
            t0 = time.perf_counter()
            res = srv.run(reqs, duration=3.0 * args.serve_duration, admit_until=args.serve_duration)
            wall = time.perf_counter() - t0
            s = summarize(res, wall)
            s["requests_arrived"] = len(reqs)
            s["peak_budget_used_gb"] = srv.peak_used / GB
            s["admission_host_ms_mean"] = 1e3 * sum(srv.admission_host_s) / max(len(srv.admission_host_s), 1)
            per[prec] = s
            del srv, res
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
        out["rates"][str(rate)] = per
    return out


def _shelf_leg(args, device):
    """The many-tracer shelf sea (20 passive tracers, tidal open boundaries):
    step time of both forms and, after ``--shelf-steps`` 3D steps, the
    per-tracer error and the compensated tracer totals of the mixed form
    against FP64."""
    import numpy as np
    import torch

    from getm_gb300 import workloads

    nx, ny, nz = (int(v) for v in args.shelf_size.split("x"))
    wl = workloads.shelf_sea(nx=nx, ny=ny, nz=nz, ntracer=20)
    cells = nx * ny * nz
    out = {"workload": f"shelf sea {nx}x{ny}x{nz}, 20 passive tracers, M2 tide on open boundaries, "
                       f"{wl.params['split_factor']} substeps per 3D step", "steps": args.shelf_steps}
    runners = {}
    for f in ("mixed", "fp64"):
        r = Runner(workloads.start_shelf_sea(wl, f, device), 3, not args.no_graph)
        ms, _ = r.timed(10)
        out[f] = {"ms_per_step": ms / 10, "value": cells * 10 / (ms / 1000.0)}
        runners[f] = r
    for r in runners.values():
        r.run_to(args.shelf_steps)
    torch.cuda.synchronize()
    a, b = runners["mixed"].sim, runners["fp64"].sim
    wet = torch.from_numpy(wl.T.mask == 1).to(device)
    errs = []
    for x, y in zip(a.tracers._tracers, b.tracers._tracers):
        xv, yv = x.all_values.double()[..., wet], y.all_values[..., wet]
        errs.append(float((xv - yv).abs().max() / yv.abs().max()))
    ta, tb = a.totals_device().tolist(), b.totals_device().tolist()
    za, zb = a.T.z.all_values[wet], b.T.z.all_values[wet]
    out.update({"steps_done": runners["mixed"].steps_done, "tracer_error_max": max(errs),
                "tracer_error_median": float(np.median(errs)),
                "tracer_totals_vs_fp64_max": max(abs(x - y) / abs(y) for x, y in zip(ta[1:], tb[1:])),
                "volume_vs_fp64": (ta[0] - tb[0]) / tb[0],
                "z_error_m": float((za - zb).abs().max()), "z_max_m": float(zb.abs().max()),
                # the elevation metric: max error over the FP64 run's range of z
                "z_error_rel_range": float((za - zb).abs().max() / (zb.max() - zb.min()))})
    del runners, a, b
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def _substep_kernel_leg(runner, peak, peak_kind):
    """Time the one-launch 2D substep (substep_2d_kernel) on the live state:
    CUDA events around every substep of two 3D steps that is not followed
    by a 3D step (one launch each), against the substep's algorithmic bytes
    (its 2D fields stay resident in L2, so the HBM figure is a reference
    point, not its bound)."""
    import torch

    from getm_gb300 import roofline

    sim = runner.sim
    if sim._split2d is None:
        return None
    if runner.steps_done % runner.period:
        runner.run_step()
    torch.cuda.synchronize()
    times = []
    for _ in range(2):
        for k in range(sim.split_factor):
            if k == sim.split_factor - 1:
                sim.advance()
                continue
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            sim.advance()
            e1.record()
            times.append((e0, e1))
        runner.steps_done += 1
        if runner.hook is not None:
            runner.hook(sim)
    torch.cuda.synchronize()
    runner.check()
    us = sorted(a.elapsed_time(b) * 1000.0 for a, b in times)
    t = us[len(us) // 2] / 1e6
    T = sim.T
    b = roofline.substep_bytes(T.nx, T.ny)
    return {"kernel": f"substep_2d_kernel<{'true' if sim.precision == 'mixed' else 'false'}>",
            "us_per_launch_median": us[len(us) // 2], "launches_timed": len(us),
            "bytes_per_launch": b, "achieved_gbs": b / t / 1e9, "peak": peak, "peak_kind": peak_kind,
            "frac_of_hbm": b / t / 1e9 / peak,
            "note": "2D fields of one plane are L2-resident; bound by FP64 pipe, barriers and latency"}


def _tracer_transport_leg(args, device, threads):
    """The plain FP64 tracer transport (120 x 100 x 30, superbee, implicit
    vertical diffusion): 500 steps on the GPU (each step one graph replay)
    against the oracle on the host cores (a sample of 50 steps)."""
    import torch

    from getm_gb300 import workloads
    from getm_gb300.simulation import TracerTransport

    wl = workloads.tracer_transport()
    nsteps = 500
    g = TracerTransport(wl, device=device)
    for _ in range(3):
        g.step()
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            g.step()
    torch.cuda.current_stream().wait_stream(stream)
    graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(nsteps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0
    out = {"workload": "tracer transport 120x100x30, dt 30 s, superbee + implicit vertical diffusion, FP64",
           "steps": nsteps, "value": wl.cells * nsteps / t, "unit": "cell-updates/s",
           "ms_per_step": 1000.0 * t / nsteps, "cuda_graph": True}
    if not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
        os.environ.setdefault("GETM_ORACLE_VARIANT", "omp" if threads > 1 else "serial")
        from oracle.models import TracerTransport as OT

        o = OT(wl)
        o.step()
        n = 50
        t0 = time.perf_counter()
        for _ in range(n):
            o.step()
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": wl.cells * n / tc, "unit": "cell-updates/s", "cores": threads,
                               "kind": "port", "sample": f"{n} steps"}
    del g, graph
    torch.cuda.synchronize()
    return out


def run_ours(args):
    import torch

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import __graft_entry__

    __graft_entry__.build()
    from getm_gb300 import roofline, workloads

    device = f"cuda:{local}"
    wl = workloads.seamount(nx=args.nx, ny=args.ny, nz=args.nz)
    nsteps = args.steps
    primary = args.precision
    forms = [primary] + ([] if args.no_compare else [f for f in ("fp64", "mixed") if f != primary])
    runners = {f: Runner(_make_sim(wl, f, device, tracer_storage=args.tracer_storage if f == "mixed" else None),
                         args.warmup, not args.no_graph) for f in forms}

    # device-timed region for each form: exactly nsteps 3D steps
    ms = {}
    clocks = None
    for f in forms:
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        m, c = runners[f].timed(nsteps, clocks_index=local if f == primary else None)
        if f == primary:
            clocks = c
        ms[f] = _max_over_ranks(m, "cuda")
    cells = wl.cells
    values = {f: _whole_job_rate(cells, nsteps, ms[f]) for f in forms}

    # end to end through the public API: before every 3D step the surface
    # forcing (taux, tauy, sp) is uploaded from pinned host memory, after
    # it the surface elevation z is read back
    e2e = {}
    for f in forms:
        r = runners[f]
        sim = r.sim
        forcing = [sim.airsea.taux, sim.airsea.tauy, sim.airsea.sp]
        host_in = [x.all_values.detach().cpu().pin_memory() for x in forcing]
        host_out = torch.empty(sim.T.z.all_values.shape, dtype=torch.float64).pin_memory()
        h2d = sum(h.numel() * h.element_size() for h in host_in)
        d2h = host_out.numel() * host_out.element_size()
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(nsteps):
            for x, h in zip(forcing, host_in):
                x.all_values.copy_(h, non_blocking=True)
            r.run_step()
            host_out.copy_(sim.T.z.all_values, non_blocking=True)
        torch.cuda.synchronize()
        dt = _max_over_ranks(time.perf_counter() - t0, "cuda")
        r.check()
        e2e[f] = {"value": _whole_job_rate(cells, nsteps, 1000.0 * dt), "unit": "cell-updates/s",
                  "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    # error of the mixed form against FP64 after the same number of 3D steps
    err = None
    if "mixed" in runners and "fp64" in runners and args.error_steps > 0 and rank == 0:
        err = _errors(wl, runners, args, device)
        for r in runners.values():
            r.check()

    peak, peak_kind = _peaks()
    roofline_kernel = _roofline(runners[primary].sim, peak, peak_kind)
    T = wl.T
    step_roof = {}
    for f in forms:
        b = roofline.step_bytes(T.nx, T.ny, T.nz, f, ntracer=2, split=wl.params["split_factor"],
                                tracer_storage=runners[f].sim.tracer_storage)
        t = ms[f] / nsteps / 1000.0
        step_roof[f] = {"bytes_per_step": b["total"], "bytes_3d": b["3d"], "bytes_2d_loop": b["2d"],
                        "achieved_gbs": b["total"] / t / 1e9, "peak": peak, "peak_kind": peak_kind,
                        "frac": b["total"] / t / 1e9 / peak}
    substep = _substep_kernel_leg(runners[primary], peak, peak_kind)
    if substep is not None:
        # the dominant kernel of the step (29 launches per 3D step)
        roofline_main = {"bound": "hbm", "achieved": substep["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": substep["frac_of_hbm"], "traffic": TRAFFIC_SUBSTEP.get(primary),
                         "kernel": substep["kernel"], "bytes_per_launch": substep["bytes_per_launch"],
                         "us_per_launch": substep["us_per_launch_median"], "peak_kind": peak_kind,
                         "note": "one 2D substep; its fields stay resident in L2, so HBM is a reference point "
                                 "(bound: FP64 pipe and grid barriers)"}
    else:
        roofline_main = roofline_kernel
    r = runners[primary]
    line = {"metric": "3D cell-updates/s", "value": values[primary], "unit": "cell-updates/s", "n_gpus": ws,
            "steps": nsteps, "warmup": max(args.warmup, 3), "ms_per_step": ms[primary] / nsteps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if primary == "mixed" else "f64", "data": "synthetic",
            "config": _config(wl, ws), "form": primary, "tracer_storage": str(r.sim.dtype_tracer).replace("torch.", ""),
            "tiles": r.sim.tiles, "cuda_graph": r.graphs is not None,
            "e2e": e2e[primary], "roofline": roofline_main, "roofline_xpass": roofline_kernel,
            "step_roofline": step_roof,
            "gpu_launches": r.launches_per_period * nsteps // r.period, "clocks": clocks,
            "split2d_status": {f: runners[f].sim.split2d_status() for f in forms}}
    if substep is not None:
        line["substep_kernel"] = substep
    if primary == "mixed" and args.column_solve and rank == 0:
        line["column_solve"] = _column_solve_leg(runners[primary].sim, device)
    for f in forms:
        if f != primary:
            line[f] = {"value": values[f], "ms_per_step": ms[f] / nsteps, "e2e": e2e[f]["value"]}
    if err is not None:
        line["error_vs_fp64"] = err
    threads = _host_threads()
    if rank == 0 and args.c1:
        line["tracer_transport"] = _tracer_transport_leg(args, device, threads)
    if rank == 0 and args.ensemble > 0:
        line["ensemble"] = _ensemble_leg(args, device)
    if rank == 0 and args.serve_rates:
        line["serving"] = _serving_leg(args, device)
    if rank == 0 and args.shelf_steps > 0:
        line["shelf_sea"] = _shelf_leg(args, device)
    if rank == 0 and not args.no_cpu_baseline and ws == 1:
        v, dt = cpu_reference(args, 2, threads)
        line["cpu_baseline"] = {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                                "sample": f"2 3D steps of the full workload ({dt:.1f} s)"}
        line["speedup_vs_cpu"] = {f"{f}_e2e": e2e[f]["value"] / v for f in forms}
        line["speedup_vs_cpu"].update({f"{f}_device": values[f] / v for f in forms})
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    args = _args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
