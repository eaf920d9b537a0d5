"""The allocation-free 2D advection split against the handle-based one.

getm_advection_2d_noalloc exists for callers that cannot let the library
call cudaMalloc - a host model whose pool allocator owns all device memory,
or a driver that must not let a library call synchronize the device.  It keeps
its work buffers in a fixed device array shared by all calls, so this test
checks, through the C ABI, that two calls in a row (the second one running on
whatever the first left in that array) give the same results as
getm_advection_2d, and that an oversized domain is refused before any work.

This file is named to be collected last, and it sets up everything it uses,
so it passes both on its own in a fresh process and after the other tests.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the same kernels run on the same inputs: results agree to the bit


def _case(seed, split, ufirst):
    import torch

    from getm_gb300.core import make_grids
    from tests.gpu_helpers import apply_state_device, random_state
    from tests.helpers import full_grid

    Th, rng = full_grid(nx=40, ny=30, nz=4, seed=seed)
    state = random_state(Th, rng, Th.nz)
    Td = make_grids(Th)
    apply_state_device(Td, state)
    u = rng.uniform(-0.5, 0.5, (Th.ny_, Th.nx_))
    v = rng.uniform(-0.5, 0.5, (Th.ny_, Th.nx_))
    u[Th.ugrid.mask == 0] = 0.0
    v[Th.vgrid.mask == 0] = 0.0
    var = rng.uniform(1.0, 2.0, (Th.ny_, Th.nx_))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return Td, dev(u), dev(v), dev(var), split, ufirst


def _run_both(Td, u, v, var, split, ufirst, dt=600.0, scheme=5):
    import torch

    from getm_gb300 import _lib

    s = torch.cuda.current_stream().cuda_stream
    # existing entry point, through an advection handle
    h = ctypes.c_void_p()
    _lib.call("getm_advection_create", scheme, Td.handle, ctypes.byref(h))
    D_ref = Td.D.all_values.clone()
    var_ref = var.clone()
    _lib.call("getm_advection_2d", h, Td.handle, Td.ugrid.handle, Td.vgrid.handle, int(ufirst), split,
              u.data_ptr(), v.data_ptr(), None, None, dt, D_ref.data_ptr(), Td.ugrid.D.all_values.data_ptr(),
              Td.vgrid.D.all_values.data_ptr(), var_ref.data_ptr(), s)
    # allocation-free entry point
    D_new = Td.D.all_values.clone()
    var_new = var.clone()
    rc = _lib.lib.getm_advection_2d_noalloc(scheme, Td.handle, Td.ugrid.handle, Td.vgrid.handle, int(ufirst), split,
                                            u.data_ptr(), v.data_ptr(), None, None, dt, D_new.data_ptr(),
                                            Td.ugrid.D.all_values.data_ptr(), Td.vgrid.D.all_values.data_ptr(),
                                            var_new.data_ptr(), s)
    assert rc == 0, f"getm_advection_2d_noalloc returned {rc}"
    torch.cuda.synchronize()
    _lib.call("getm_advection_finalize", h)
    return (var_new.cpu().numpy(), var_ref.cpu().numpy()), (D_new.cpu().numpy(), D_ref.cpu().numpy())


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_two_calls_in_a_row_match_the_handle_version():
    # first call: HALF split (3 passes, ends with a copy back); second call:
    # different domain, inputs and split, reusing the shared scratch array
    for seed, split, ufirst in ((7, 2, False), (8, 3, True)):
        Td, u, v, var, split, ufirst = _case(seed, split, ufirst)
        (vn, vr), (dn, dr) = _run_both(Td, u, v, var, split, ufirst)
        assert _rel(vn, vr) <= RTOL
        assert _rel(dn, dr) <= RTOL
        # the advection did something
        assert _rel(vn, var.cpu().numpy()) > 0.0


def test_oversized_domain_is_refused():
    from getm_gb300 import _lib

    big = ctypes.c_void_p()
    # 1100 x 1000 interior + halos: more points than the fixed scratch holds
    assert _lib.lib.getm_create_grid(1, 1100, 1, 1000, 1, 1, 2, 2, ctypes.byref(big)) == 0
    rc = _lib.lib.getm_advection_2d_noalloc(5, big, big, big, 0, 1, None, None, None, None, 1.0, 1, 1, 1, 1, None)
    assert rc == 6  # GETM_ERR_TOO_LARGE, before any device work
    _lib.lib.getm_grid_finalize(big)
