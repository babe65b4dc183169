"""dgsw_step_noalloc: stepping for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc while they step -- a host framework that
owns a fixed device-memory budget and only lends plug-ins the buffers it has
placed, or a caller that must not trigger cudaMalloc's device-wide
synchronisation.  dgsw_step_noalloc keeps all of its scratch in one fixed
device array inside the library.  These tests call it through the C ABI and
check it, for two calls in a row (the second call reuses the array the first
one left behind):
  - against the handle-based dgsw_step on the same state,
  - against the CPU oracle's SSP-RK3 evolution directly,
  - with gamma2 != 0 and on a non-default CUDA stream,
  - and that the device's free memory is the same before and after calls once
    the library's device code is loaded (nothing is allocated per call).
The file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes
import math

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, DgEvolution, DgswBrick

pytestmark = pytest.mark.gpu
RTOL = 1e-12  # the FP64 per-step tolerance used for the plain path


def _brick(elements, lower=(0.0, 0.0, 0.0), upper=(2 * math.pi,) * 3):
    b = DgswBrick()
    b.lower[:] = list(lower)
    b.upper[:] = list(upper)
    b.elements[:] = list(elements)
    return b


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _call(L, brick, n, gamma2, u, steps, dt, stream_ptr=None):
    rc = L.dgsw_step_noalloc(ctypes.byref(brick), n, gamma2, u.data_ptr(), steps, dt,
                             stream_ptr)
    assert rc == 0, L.dgsw_noalloc_last_error()


@pytest.mark.parametrize("elements,points", [((4, 4, 4), 6), ((3, 2, 4), 5)])
def test_noalloc_matches_handle_step_two_calls(elements, points):
    import torch
    L = dgsw.lib()
    n, dt, steps = points, 1e-3, 3
    params = np.array([[1.0, 0.8, 2.0, 3.0, 4.0]])
    with DgEvolution([Brick(elements)], n) as ev:
        ev.set_initial_data("gaussian", params)
        u0 = ev.get_state()
        ev.step(steps, dt)
        ref1 = ev.get_state()
        ev.step(steps, dt)
        ref2 = ev.get_state()
    brick = _brick(elements)
    u = torch.tensor(u0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _call(L, brick, n, 0.0, u, steps, dt)
    torch.cuda.synchronize()
    got1 = u.cpu().numpy()
    _call(L, brick, n, 0.0, u, steps, dt)
    torch.cuda.synchronize()
    got2 = u.cpu().numpy()
    assert _rel(got1, ref1) <= RTOL
    assert _rel(got2, ref2) <= RTOL


@pytest.mark.parametrize("gamma2", [0.0, 1.5])
def test_noalloc_matches_oracle_on_a_side_stream(oracle, gamma2):
    """Two calls in a row on a non-default stream against the oracle's own
    SSP-RK3 evolution (Rk3HesthavenSsp.cpp:63-80 restated on the CPU), and the
    device's free memory unchanged across the calls."""
    import torch
    L = dgsw.lib()
    elements, n, dt, steps = (3, 4, 2), 6, 2e-3, 2
    bricks = [Brick(elements)]
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1.0, 1.0, 1.0])
    ref1 = oracle.evolve(bricks, n, u0, dt, steps, gamma2=gamma2)
    ref2 = oracle.evolve(bricks, n, ref1, dt, steps, gamma2=gamma2)
    brick = _brick(elements)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        u = torch.tensor(u0, dtype=torch.float64, device="cuda")
    side.synchronize()
    # load the library's device code (and its fixed array) before measuring
    warm = u.clone()
    torch.cuda.synchronize()
    _call(L, brick, n, gamma2, warm, 1, dt, side.cuda_stream)
    side.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _call(L, brick, n, gamma2, u, steps, dt, side.cuda_stream)
    side.synchronize()
    got1 = u.cpu().numpy()
    free1, _ = torch.cuda.mem_get_info()
    _call(L, brick, n, gamma2, u, steps, dt, side.cuda_stream)
    side.synchronize()
    got2 = u.cpu().numpy()
    free2, _ = torch.cuda.mem_get_info()
    assert _rel(got1, ref1) <= RTOL
    assert _rel(got2, ref2) <= RTOL
    assert free0 == free1 == free2, (free0, free1, free2)


def test_noalloc_rejects_bricks_beyond_the_fixed_scratch():
    import torch
    L = dgsw.lib()
    assert L.dgsw_noalloc_scratch_bytes() == 32 * 1024 * 1024
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    too_big = _brick((16, 16, 16))  # 4096 elements x 8^3 points
    rc = L.dgsw_step_noalloc(ctypes.byref(too_big), 8, 0.0, u.data_ptr(), 1, 1e-3, None)
    assert rc == -1
    assert b"32 MiB" in L.dgsw_noalloc_last_error()
    # host memory is refused before anything is launched
    host = np.zeros(5 * 8 * 8)
    rc = L.dgsw_step_noalloc(ctypes.byref(_brick((2, 2, 2))), 2, 0.0, host.ctypes.data, 1,
                             1e-3, None)
    assert rc == -1
    assert b"device memory" in L.dgsw_noalloc_last_error()
