"""Events::ObserveNorms on the device vs the oracle's restatement.

Max / Min are exact; the sums are FP64 with a different summation order, so
they agree to 1e-13 relative.  The plane-wave error norms are checked against
the oracle's norms of (state - analytic solution)."""
import math

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick, CurvedDgEvolution, DgEvolution, Shell

pytestmark = pytest.mark.gpu


def _check(raw, ref):
    for v in range(5):
        assert raw[5 * v] == ref[5 * v] and raw[5 * v + 1] == ref[5 * v + 1]
        for m in (2, 3, 4):
            assert abs(raw[5 * v + m] - ref[5 * v + m]) <= 1e-13 * max(1.0, abs(ref[5 * v + m]))
    assert raw[25] == ref[25]
    assert abs(raw[26] - ref[26]) <= 1e-13 * ref[26]


def test_norms_flat_uniform_and_mixed_extents(oracle):
    rng = np.random.default_rng(1)
    for bricks, pts in (([Brick((3, 2, 4))], 6),
                        ([Brick((2, 2, 3)), Brick((1, 2, 2), (0, 0, 0), (1, 2, 3))],
                         rng.integers(4, 11, size=16).astype(np.int32))):
        en = oracle.elem_points(bricks, pts)
        u = rng.uniform(-2, 2, int(oracle.offsets(en)[-1]))
        with DgEvolution(bricks, pts) as ev:
            ev.set_state(u)
            got = ev.observe_norms()
        _check(got["raw"], oracle.observe_norms(bricks, pts, u))


def test_norms_curved_shell(oracle):
    s = oracle.shell(1.9, 20.0, 1, 2, 8)
    u = oracle.shell_initial_data(s, 8.0, 1.0)
    with CurvedDgEvolution(Shell(1.9, 20.0, 1, 2), 8) as ev:
        ev.set_state(u.ravel())
        got = ev.observe_norms()
    ref = oracle.shell_observe_norms(s, u)
    _check(got["raw"], ref)
    assert abs(got["Volume"] - 4.0 / 3.0 * math.pi * (20.0 ** 3 - 1.9 ** 3)) < 1e-8


def test_plane_wave_error_norms(oracle):
    bricks = [Brick((4, 4, 4))]
    n, dt, steps = 6, 1e-3, 50
    k = [1.0, 1.0, 1.0]
    with DgEvolution(bricks, n) as ev:
        ev.set_initial_data("plane_wave", k)
        ev.step(steps, dt)
        got = ev.observe_plane_wave_errors(k, steps * dt)
        state = ev.get_state()
    exact = oracle.initial_data(bricks, n, "plane_wave", k, t=steps * dt)
    _check(got["raw"], oracle.observe_norms(bricks, n, state, subtract=exact))
    # discretisation error of the 4^3 x 6^3 plane wave after 50 steps
    assert got["L2Norm(Error(Psi))"] < 5e-3


def test_norms_survive_sample_setup(oracle):
    # setting sample points must not release the handle's other device tables
    bricks = [Brick((2, 2, 2))]
    with DgEvolution(bricks, 8) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        a = ev.observe_norms()["raw"].copy()
        ev.set_samples(np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 1.5]]))
        ev.set_exponential_filter(36.0, 8)
        b = ev.observe_norms()["raw"]
        ev.set_samples(np.array([[0.5, 0.5, 0.5]]))
        c = ev.observe_norms()["raw"]
        ev.step(2, 1e-3)
    assert np.array_equal(a, b) and np.array_equal(a, c)
