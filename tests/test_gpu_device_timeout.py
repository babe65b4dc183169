"""Failure detection of the device-side waits, without a GPU fault.

The mixed-precision pipeline waits on mbarriers for its staged copies with a
wall-clock bound.  Here the same wait routine runs on a barrier that nothing
completes, with a 50 ms bound: the kernel gives up, records the error word and
returns, the library reports DGSW_ERR_DEVICE_TIMEOUT, and the handle (and the
CUDA context) stay usable for the next step."""
import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, DgEvolution

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_handle_survives(oracle):
    bricks = [Brick((2, 2, 2))]
    n = 8
    with DgEvolution(bricks, n, precision=dgsw.PRECISION_MIXED) as ev:
        st = ev.check_device_timeout(0.05)
        assert st == -6  # DGSW_ERR_DEVICE_TIMEOUT
        assert "timed out" in dgsw.lib().dgsw_last_error(ev.handle).decode()
        # the error word was cleared; the next steps run and agree with FP64
        u = oracle.initial_data(bricks, n, "plane_wave", [1.0, 1.0, 1.0])
        ev.set_state(u)
        ev.step(5, 1e-3)
        got = ev.get_state()
    ref = oracle.evolve(bricks, n, u, 1e-3, 5)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6


def test_timeout_limit_validated():
    with DgEvolution([Brick((1, 1, 1))], 4) as ev:
        with pytest.raises(dgsw.DgswError):
            dgsw._check(dgsw.lib().dgsw_check_device_timeout(ev.handle, 0.0), ev.handle)
