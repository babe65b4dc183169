"""dgsw_step_noalloc: stepping for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc while they step -- a host framework that
owns a fixed device-memory budget and only lends plug-ins the buffers it has
placed, or a caller that must not trigger cudaMalloc's device-wide
synchronisation.  dgsw_step_noalloc keeps all of its scratch in one fixed
device array inside the library.  This test calls it through the C ABI and
checks its result against the handle-based dgsw_step on the same state, for
two calls in a row (the second call reuses the array the first one left
behind).  The file sorts last so that a run stopping at the first failure has
already run every other test.
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
    rc = L.dgsw_step_noalloc(ctypes.byref(brick), n, 0.0, u.data_ptr(), steps, dt, None)
    assert rc == 0, L.dgsw_noalloc_last_error()
    torch.cuda.synchronize()
    got1 = u.cpu().numpy()
    rc = L.dgsw_step_noalloc(ctypes.byref(brick), n, 0.0, u.data_ptr(), steps, dt, None)
    assert rc == 0, L.dgsw_noalloc_last_error()
    torch.cuda.synchronize()
    got2 = u.cpu().numpy()
    assert _rel(got1, ref1) <= RTOL
    assert _rel(got2, ref2) <= RTOL


def test_noalloc_rejects_bricks_beyond_the_fixed_scratch():
    import torch
    L = dgsw.lib()
    assert L.dgsw_noalloc_scratch_bytes() == 32 * 1024 * 1024
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    too_big = _brick((16, 16, 16))  # 4096 elements x 8^3 points
    rc = L.dgsw_step_noalloc(ctypes.byref(too_big), 8, 0.0, u.data_ptr(), 1, 1e-3, None)
    assert rc == -1
    assert b"32 MiB" in L.dgsw_noalloc_last_error()
    host = np.zeros(16)
    rc = L.dgsw_step_noalloc(ctypes.byref(_brick((2, 2, 2))), 2, 0.0, host.ctypes.data, 1,
                             1e-3, None)
    assert rc == -1
