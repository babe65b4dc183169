"""dgsw_step_host: steps of a host-resident state with the copies overlapped
chunk by chunk.  The chunked launches run the same per-element arithmetic as
dgsw_step, so the result must be bit-identical to set_state + step +
get_state."""
import math

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick, DgEvolution

pytestmark = pytest.mark.gpu


def _state(ev, params=(1.0, 0.5, math.pi, math.pi, math.pi)):
    ev.set_initial_data("gaussian", list(params))
    ev.step(2, 2e-4)  # a state with structure in every variable
    return ev.get_state()


@pytest.mark.parametrize("elements,n,steps", [((32, 32, 32), 8, 1), ((32, 32, 32), 8, 2),
                                              ((16, 20, 24), 6, 5), ((20, 16, 16), 4, 3),
                                              ((4, 4, 4), 6, 2)])
def test_step_host_bit_identical(elements, n, steps):
    bricks = [Brick(elements)]
    with DgEvolution(bricks, n) as ev:
        u0 = _state(ev)
        ev.set_state(u0)
        ev.step(steps, 2e-4)
        want = ev.get_state()
        import torch
        host = torch.empty(ev.state_size, dtype=torch.float64, pin_memory=True).numpy()
        host[:] = u0
        ev.step_host(host, steps, 2e-4)
        assert np.array_equal(host, want)
        # the handle's device state is the stepped state too
        assert np.array_equal(ev.get_state(), want)


def test_step_host_pageable_and_two_bricks():
    bricks = [Brick((16, 16, 12)), Brick((12, 16, 16), (0.0, 0.0, 0.0), (1.0, 2.0, 3.0))]
    with DgEvolution(bricks, 5) as ev:
        u0 = _state(ev, (1.0, 0.5, math.pi, math.pi, math.pi, 1.0, 0.3, 0.5, 1.0, 1.5))
        assert np.all(np.isfinite(u0))
        ev.set_state(u0)
        ev.step(3, 2e-4)
        want = ev.get_state()
        host = u0.copy()  # pageable numpy memory
        ev.step_host(host, 3, 2e-4)
        assert np.array_equal(host, want)


def test_step_host_graph_reuse_and_new_dt():
    # pinned buffers replay a captured graph per (pointer, dt)
    import torch
    with DgEvolution([Brick((32, 16, 16))], 6) as ev:
        u0 = _state(ev)
        ev.set_state(u0)
        ev.step(3, 2e-4)
        want = ev.get_state()
        host = torch.empty(ev.state_size, dtype=torch.float64, pin_memory=True).numpy()
        host[:] = u0
        for _ in range(3):
            ev.step_host(host, 1, 2e-4)
        assert np.array_equal(host, want)
        ev.set_state(u0)
        ev.step(1, 1e-4)
        want = ev.get_state()
        host[:] = u0
        ev.step_host(host, 1, 1e-4)
        assert np.array_equal(host, want)
