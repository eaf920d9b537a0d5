"""ctypes binding of the C ABI declared in include/getm_gb300.h.

The product path has exactly one implementation: the sm_103a CUDA library.
If ``libgetm_gb300.so`` is missing this module raises on import - there is no
CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading
from ctypes import c_double, c_int, c_void_p
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("GETM_GB300_LIB", _HERE / "libgetm_gb300.so"))

GETM_OK = 0
GETM_MAX_TOTALS = 16      # include/getm_gb300.h
GETM_TOTALS_BLOCKS = 608  # include/getm_gb300.h
ERRORS = {
    1: "invalid argument",
    2: "CUDA launch/runtime error",
    3: "vertical advection exceeded itersmax sub-steps",
    4: "too many layers for a column kernel",
    5: "device work-buffer allocation failed",
    6: "domain larger than the fixed scratch of an allocation-free call",
}

if not LIB_PATH.exists():
    raise ImportError(
        f"{LIB_PATH} not found: build the CUDA library first "
        "(python -c 'import __graft_entry__ as g; g.build()')"
    )

lib = ctypes.CDLL(str(LIB_PATH))

# argument codes: i int, d double, p pointer (device array / handle / host array), s stream
_SIGS = {
    "getm_create_grid": "iiiiiiiip",
    "getm_grid_finalize": "p",
    "getm_grid_set_array": "pcp",
    "getm_grid_float_metrics": "ps",
    "getm_advection_create": "ipp",
    "getm_advection_finalize": "p",
    "getm_advection_uv_calculate": "iipppppdppps",
    "getm_advection_w_calculate": "ppppdpps",
    "getm_advection_apply_3d_batch": "ppppippppppdpppips",
    "getm_advection_2d": "ppppiippppdpppps",
    "getm_advection_2d_mixed": "ppppiippppdpppps",
    "getm_advection_get_status": "ps",
    "getm_advection_2d_noalloc": "ipppiippppdpppps",
    "getm_advection_uv_pass": "iipppppdpppipps",
    "getm_advection_uv_pass_f32": "iipppppdpppipps",
    "getm_advection_uv_pass_f64s": "iipppppdpppipps",
    "getm_vertical_diffusion_create": "pp",
    "getm_vertical_diffusion_finalize": "p",
    "getm_vertical_diffusion_prepare": "piiidpddppps",
    "getm_vertical_diffusion_apply": "piiipppppps",
    "getm_vertical_diffusion_batch": "iiippddppippppps",
    "getm_grid_interp_x": "iiippis",
    "getm_grid_interp_y": "iiippis",
    "getm_grid_interp_z": "iiiippis",
    "getm_grid_interp_xy": "iiiiippiis",
    "getm_momentum_diffusion": "ppppppippppppdpps",
    "getm_thickness2center_depth": "iiiiiiippps",
    "getm_thickness2vertical_coordinates": "iiippppps",
    "getm_alpha": "ipddpps",
    "getm_elevation2depth": "ippdpps",
    "getm_multiply_add": "ippds",
    "getm_advance_surface_elevation": "iiiippppppppds",
    "getm_surface_pressure_gradient": "iiiiiippppppppdpps",
    "getm_shear_frequency2": "iiiiiiipppppppps",
    "getm_shear_frequency2_f32": "iiiiiiipppppppps",
    "getm_vertical_advection_to_sources": "iiiiipppppps",
    "getm_update_gvc": "iiidpdippps",
    "getm_surface_pressure_gradient_mixed": "iiiiiippppppppdpps",
    "getm_horizontal_diffusion": "iiiiiippppppppppdpps",
    "getm_bottom_friction": "iippppppdpis",
    "getm_bottom_friction_mixed": "iippppppdpis",
    "getm_update_depth_2d": "iidd" + "p" * 25 + "s",
    "getm_update_depth_2d_mixed": "iidd" + "p" * 25 + "s",
    "getm_momentum_2d_velocities": "iii" + "p" * 16 + "s",
    "getm_momentum_2d_friction": "iii" + "p" * 12 + "s",
    "getm_coriolis_2d": "iiiipppis",
    "getm_coriolis_2d_mixed": "iiiipppis",
    "getm_advance_2d_transport_mixed": "iiiippppppppppppppdps",
    "getm_accumulate_2d": "lpppps",
    "getm_surface_elevation_fused": "iiiipppppppppds",
    "getm_split2d_substep": "piiiiiiiidddppppippppis",
    "getm_update_depth_3d": "piiis",
    "getm_transport_3d_finish": "iiipppppps",
    "getm_transport_3d_finish_f32": "iiipppppps",
    "getm_velocities_3d": "lpppppps",
    "getm_momentum_3d_advection_inputs": "iiippppppppppps",
    "getm_momentum_3d_advection_inputs_f32": "iiippppppppppps",
    "getm_coriolis_3d": "iiiiipppis",
    "getm_coriolis_3d_f32": "iiiiipppis",
    "getm_substep_batch_create": "iip",
    "getm_substep_batch_set": "piiipiiiiiiidddppppippppi",
    "getm_substep_batch_upload": "p",
    "getm_substep_batch_participants": "pip",
    "getm_substep_batch_launch": "piips",
    "getm_substep_batch_finalize": "p",
    "getm_mean_transports": "lppdpps",
    "getm_slow_friction": "lpppppppps",
    "getm_velocities_3d_bottom_f32": "llpppppppps",
    "getm_keps_default_params": "p",
    "getm_keps_advance": "iiiiipdpppppppppppppps",
    "getm_keps_advance_f32": "iiiiipdpppppppppppppps",
    "getm_tune_set": "ii",
    "getm_tune_get": "ip",
    "getm_coriolis_espelid": "iiiiipppppppis",
    "getm_coriolis_espelid_f32": "iiiiipppppppis",
    "getm_buoyancy_frequency": "iiipppppps",
    "getm_buoyancy_frequency_f32": "iiipppppps",
    "getm_buoyancy_frequency_f64s": "iiipppppps",
    "getm_column_sums": "iiiipppppppps",
    "getm_column_sums_f32": "iiiipppppppps",
    "getm_velocities_3d_f32": "lpppppps",
    "getm_open_boundary_elevation": "iiipppppppppppppdps",
    "getm_open_boundary_tracers": "iiiiiiippppppipps",
    "getm_open_boundary_tracers_f32": "iiiiiiippppppipps",
    "getm_mirror": "ippilpps",
    "getm_mirror_f32": "ippilpps",
    "getm_open_boundary_depth": "ippppppddppps",
    "getm_collect_3d_momentum_sources": "iiiiipppppppppppdpps",
    "getm_advance_2d_transport": "iiiippppppppppppppdps",
    "getm_w_momentum_3d": "iiiiiiippppppppdps",
    "getm_shear_frequency": "iiiiiiipppppps",
    "getm_surface_shear_velocity": "iiiiiipppps",
    "getm_bottom_shear_velocity": "iiiiiipppppppppps",
    "getm_reconstruct_transport_change": "iiiiiiipppds",
    "getm_blumberg_mellor": "iiiiiiipppppppppps",
    "getm_shchepetkin_mcwilliams": "iiiiiiipppppppppppps",
    "getm_shchepetkin_mcwilliams_mixed": "iiiiiiipppppppppppps",
    "getm_density_buoyancy": "ippppps",
    "getm_launch_count": "p",
    "getm_graph_launch": "ps",
    "getm_advance_time": "pds",
    "getm_stream_create": "is",
    "getm_stream_destroy": "s",
    "getm_advection_apply_3d_batch_f32": "ppppippppppdpppips",
    "getm_advection_apply_3d_batch_f64s": "ppppippppppdpppips",
    "getm_vertical_diffusion_batch_f32": "iiippddppippppps",
    "getm_vertical_diffusion_batch_f64s": "iiippddppippppps",
    "getm_grid_interp_x_f32": "iiippis",
    "getm_grid_interp_y_f32": "iiippis",
    "getm_grid_interp_z_f32": "iiiippis",
    "getm_grid_interp_xy_f32": "iiiiippiis",
    "getm_collect_3d_momentum_sources_f32": "iiiiipppppppppppdpps",
    "getm_w_momentum_3d_f32": "iiiiiiippppppppdps",
    "getm_shear_frequency_f32": "iiiiiiipppppps",
    "getm_reconstruct_transport_change_f32": "iiiiiiipppds",
    "getm_blumberg_mellor_f32": "iiiiiiipppppppppps",
    "getm_shchepetkin_mcwilliams_f32": "iiiiiiipppppppppppps",
    "getm_density_buoyancy_f32": "ippppps",
    "getm_density_buoyancy_f64s": "ippppps",
    "getm_domain_totals": "iiiiiiippppippps",
    "getm_domain_totals_f32": "iiiiiiippppippps",
}
_CT = {"i": c_int, "l": ctypes.c_longlong, "d": c_double, "p": c_void_p, "s": c_void_p, "c": ctypes.c_char_p}

# The same library bound a second time with the interpreter lock held during
# the call.  Almost every entry point only checks arguments and enqueues
# work on a stream (microseconds); releasing and re-taking the lock around
# each of them lets another Python thread (the serving loop's step issue, or
# its admission worker) take the lock, and the caller then waits up to a
# whole switch interval to continue: thousands of such calls in a domain's
# set-up cost seconds.  Calls that may block (device synchronisation,
# allocation, synchronous copies) release the lock as usual.
_plib = ctypes.PyDLL(str(LIB_PATH))
_BLOCKING = frozenset({
    "getm_advection_create", "getm_advection_finalize", "getm_vertical_diffusion_create",
    "getm_vertical_diffusion_finalize", "getm_grid_finalize", "getm_advection_get_status",
    "getm_substep_batch_create", "getm_substep_batch_upload", "getm_substep_batch_finalize",
    "getm_grid_float_metrics", "getm_stream_create", "getm_stream_destroy",
})

for _name, _sig in _SIGS.items():
    for _l in (lib, _plib):
        _f = getattr(_l, _name)
        _f.argtypes = [_CT[c] for c in _sig]
        _f.restype = c_int
_CALL = {n: getattr(lib if n in _BLOCKING else _plib, n) for n in _SIGS}

EXPORTED = tuple(_SIGS)


class GetmError(RuntimeError):
    def __init__(self, name, code):
        super().__init__(f"{name} failed with status {code} ({ERRORS.get(code, 'unknown')})")
        self.code = code


# Handles whose owner was garbage-collected.  Their finalizers free device
# memory, which must not happen while a CUDA graph is being captured (on any
# thread, in the default capture mode), and a destructor can run at any
# allocation, on any thread.  So they are queued and released by the next
# library call made on a stream that is not capturing.
_pending_release = []


# Graph captures in progress on any host thread (capture_started/ended),
# e.g. a serving admission worker recording a new request while the main
# loop keeps issuing steps: no handle is finalized meanwhile (freeing device
# memory waits for the whole device, which an ongoing capture forbids).
_captures = 0
_captures_lock = threading.Lock()


def capture_started() -> None:
    global _captures
    with _captures_lock:
        _captures += 1


def capture_ended() -> None:
    global _captures
    with _captures_lock:
        _captures -= 1


def _capturing() -> bool:
    if _captures:
        return True
    try:
        import torch

        return torch.cuda.is_available() and torch.cuda.is_current_stream_capturing()
    except Exception:
        return False


def release(finalizer: str, handle) -> None:
    """Queue a library handle for finalization (see _pending_release)."""
    _pending_release.append((finalizer, handle))


def _flush_releases() -> None:
    if _capturing():
        return
    while _pending_release:
        finalizer, handle = _pending_release.pop()
        getattr(lib, finalizer)(handle)


# Threads whose library calls release the interpreter lock whatever the entry
# point (a serving admission worker): a call there can block (first-use
# allocation, module loading on a busy device) while another thread must
# keep issuing steps.
_tls = threading.local()


def release_gil_in_this_thread(flag: bool = True) -> None:
    """Make every library call of the calling thread release the interpreter
    lock (``flag``) or use the default per entry point."""
    _tls.release = flag


def call(name: str, *args) -> int:
    """Call an entry point; raise GetmError on a non-zero status."""
    if _pending_release:
        _flush_releases()
    f = getattr(lib, name) if getattr(_tls, "release", False) else _CALL[name]
    rc = f(*args)
    if rc != GETM_OK:
        raise GetmError(name, rc)
    return rc


def graph_launch(graph_exec: int, stream: int) -> None:
    """Launch an instantiated CUDA graph on a stream (getm_graph_launch).  No
    queued handle is finalized here: this is the call a loop makes while
    another thread may be capturing."""
    rc = _CALL["getm_graph_launch"](graph_exec, stream)
    if rc != GETM_OK:
        raise GetmError("getm_graph_launch", rc)


def own_stream(device, priority: int = 0):
    """A torch stream (ExternalStream) over a CUDA stream created for the
    caller alone (getm_stream_create), never one of torch's pooled streams;
    destroyed when the returned object is collected."""
    import torch

    with torch.cuda.device(device):
        h = c_void_p()
        call("getm_stream_create", int(priority), ctypes.byref(h))
    s = torch.cuda.ExternalStream(h.value, device=device)
    import weakref

    weakref.finalize(s, lib.getm_stream_destroy, h.value)
    return s


def ptr(t) -> int | None:
    """Device pointer of a torch tensor (None passes NULL)."""
    if t is None:
        return None
    return t.data_ptr()


def ptr_array(ptrs):
    """Host array of device pointers (for the batched entry points)."""
    arr = (c_void_p * len(ptrs))(*[p if p is not None else None for p in ptrs])
    return arr


def launch_count() -> int:
    """Kernel launches issued by libgetm_gb300 so far in this process."""
    n = ctypes.c_ulonglong(0)
    call("getm_launch_count", ctypes.byref(n))
    return int(n.value)


def stream_handle(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
