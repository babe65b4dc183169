"""Mixed-precision CUDA path (FP32 split-product contractions, FP64 state and
step accumulation) against the FP64 oracle and the plain FP64 CUDA path.

Tolerances: the mixed right-hand side to 1e-6 relative (max-norm per
variable: it is rounded to FP32 once); whole evolutions to <= 1e-6 relative
L2 against the FP64 oracle, the target the mixed path is specified to.
"""
import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, DgEvolution, PRECISION_MIXED, PRECISION_FP64

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_mixed_rhs_matches_oracle(oracle, n):
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (1.0, 1.5, 2.0))]
    rng = np.random.default_rng(n)
    u = oracle.initial_data(bricks, n, "gaussian", oracle.gaussian_params(1, width=0.7,
                                                                         center=(0.4, 0.8, 1.1)))
    u += 0.1 * rng.uniform(-1, 1, u.size)  # rough parts exercise the face jumps
    ref = oracle.rhs(bricks, n, u)
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as ev:
        got = ev.rhs(u)
    per_var = []
    E = len(u) // (5 * n ** 3)
    a = got.reshape(E, 5, -1)
    b = ref.reshape(E, 5, -1)
    for v in range(5):
        per_var.append(np.max(np.abs(a[:, v] - b[:, v])) / np.max(np.abs(b[:, v])))
    assert max(per_var) <= 1e-6, per_var


def test_mixed_substeps_match_oracle(oracle):
    bricks = [Brick((4, 4, 4))]
    n, dt = 6, 1e-3
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        cur = u0
        for k in range(3):
            ref = oracle.rk3_substep(k, dt, u0, cur, oracle.rhs(bricks, n, cur))
            ev.substep(k, dt)
            got = ev.get_state()
            # the state error is the FP32 rounding of an O(dt) increment
            assert rel_linf(got, ref) <= 1e-9, k
            cur = ref


def test_mixed_config1_full_run(oracle):
    # The 4^3 x 6^3 plane-wave case for 200 steps: mixed vs the FP64 oracle (rel L2 <= 1e-6)
    bricks = [Brick((4, 4, 4))]
    n, dt, steps = 6, 1e-3, 200
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        ev.step(steps, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, n, u0, dt, steps)
    err = rel_l2(got, ref)
    assert err <= 1e-6, err


def test_mixed_vs_fp64_config2_size():
    # The Gaussian-pulse grid (32^3 x 8^3, Gaussian pulse, dt 2e-4) over its full 500 steps:
    # mixed vs the plain FP64 CUDA path (which matches the oracle to 1e-12 per step)
    bricks = [Brick((32, 32, 32))]
    n, dt, steps = 8, 2e-4, 500
    params = np.array([[1.0, 0.5, np.pi, np.pi, np.pi]])
    with DgEvolution(bricks, n, precision=PRECISION_FP64) as a:
        a.set_initial_data("gaussian", params)
        a.step(steps, dt)
        ua = a.get_state()
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as b:
        b.set_initial_data("gaussian", params)
        b.step(steps, dt)
        ub = b.get_state()
    err = rel_l2(ub, ua)
    assert err <= 1e-6, err


def test_mixed_graph_chunks_equal_single_steps(oracle):
    bricks = [Brick((2, 2, 2))]
    n, dt = 5, 1e-3
    u0 = oracle.initial_data(bricks, n, "gaussian", oracle.gaussian_params(1, width=1.0))
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        ev.step(20, dt)
        a = ev.get_state()
        ev.set_state(u0)
        for _ in range(20):
            ev.step(1, dt)
        b = ev.get_state()
    np.testing.assert_array_equal(a, b)


def test_mixed_rejects_gamma2():
    with pytest.raises(dgsw.DgswError) as ei:
        DgEvolution([Brick((2, 2, 2))], 4, precision=PRECISION_MIXED, gamma2=1.0)
    assert ei.value.status == -3


@pytest.mark.parametrize("n", [6, 8])
def test_mixed_pipe_launch_shapes_agree(oracle, n):
    # the pipelined kernel's two launch shapes (dgsw_tune): same bits, and
    # both within the mixed bar of the FP64 oracle
    bricks = [Brick((4, 4, 3))]
    dt, steps = 1e-3, 30
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    ref = oracle.evolve(bricks, n, u0, dt, steps)
    out = []
    with DgEvolution(bricks, n, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        info = ev.tune()
        assert info["family"] == "mixed_pipe"
        assert np.array_equal(ev.get_state(), u0)
        assert all(ms > 0 for ms in info["ms_per_step"])
        for v in range(len(info["ms_per_step"])):
            assert ev.tune(force_variant=v)["variant"] == v
            ev.set_state(u0)
            ev.step(steps, dt)
            out.append(ev.get_state())
    for got in out:
        assert rel_l2(got, ref) <= 1e-6
    np.testing.assert_array_equal(out[0], out[1])
