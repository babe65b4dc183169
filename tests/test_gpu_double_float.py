"""Double-float precision (FP64 state, hi + lo FP32 arithmetic, the step as its
Taylor polynomial) against the FP64 oracle and the FP64 GPU path.

Tolerance: the bar of the plain FP64 path, <= 1e-12 relative per step (max
norm of the difference over the max norm of the oracle field, per
variable); over 200 steps of config 1, 200 x that bar, as for FP64.  The
double-float increments keep ~44 bits, so the measured differences are
~1e-14.
"""
import numpy as np
import pytest

from spectre_gb300.dgsw import (PRECISION_DOUBLE_FLOAT, PRECISION_FP64, Brick, DgEvolution,
                                DgswError)

from test_gpu_parity_fp64 import RTOL, random_state, rel_err_per_var

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_one_step_random_state_all_extents(oracle, n):
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (1.0, 2.0, 1.5))]
    u = random_state(np.random.default_rng(100 + n), bricks, n, oracle)
    dt = 2e-3 / n
    ref = oracle.evolve(bricks, n, u, dt, 1)
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        ev.set_state(u)
        ev.step(1, dt)
        got = ev.get_state()
    assert rel_err_per_var(got, ref, oracle.elem_points(bricks, n)) <= RTOL


@pytest.mark.parametrize("n", [3, 5, 8, 11])
def test_gamma2_steps_match_oracle(oracle, n):
    # constraint damping: the gamma2 (d_i Psi - Phi_i) term and the faces'
    # w = Pi - s Phi - gamma2 Psi in double-float
    bricks = [Brick((2, 3, 2), (0.0, 0.0, 0.0), (1.5, 2.0, 1.0))]
    gamma2 = 1.5
    u = random_state(np.random.default_rng(200 + n), bricks, n, oracle)
    dt = 2e-3 / n
    ref = oracle.evolve(bricks, n, u, dt, 2, gamma2=gamma2)
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT, gamma2=gamma2) as ev:
        ev.set_state(u)
        ev.step(2, dt)
        got = ev.get_state()
    assert rel_err_per_var(got, ref, oracle.elem_points(bricks, n)) <= 2 * RTOL


def test_multi_brick_steps(oracle):
    bricks = [Brick((2, 3, 2)), Brick((2, 2, 2), (0.0, 0.0, 0.0), (3.0, 2.0, 1.0))]
    n, dt = 5, 1e-3
    u = random_state(np.random.default_rng(7), bricks, n, oracle)
    ref = oracle.evolve(bricks, n, u, dt, 3)
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        ev.set_state(u)
        ev.step(3, dt)
        got = ev.get_state()
    assert rel_err_per_var(got, ref, oracle.elem_points(bricks, n)) <= 3 * RTOL


def test_config1_full_run_vs_oracle_and_analytic(oracle):
    bricks = [Brick((4, 4, 4))]
    n, dt, steps = 6, 1e-3, 200
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        ev.set_state(u0)
        ev.step(steps, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, n, u0, dt, steps)
    assert rel_err_per_var(got, ref, [n] * 64) <= steps * RTOL
    ua = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1], t=dt * steps)
    assert np.max(np.abs(got - ua)) < 5e-3


def test_full_size_close_to_fp64():
    # 32^3 x 8^3 Gaussian pulse, 10 steps: double-float against the FP64 GPU path
    bricks = [Brick((32, 32, 32))]
    n, dt = 8, 2e-4
    params = np.array([[1.0, 0.5, np.pi, np.pi, np.pi]])
    states = []
    for prec in (PRECISION_FP64, PRECISION_DOUBLE_FLOAT):
        with DgEvolution(bricks, n, precision=prec) as ev:
            ev.set_initial_data("gaussian", params)
            ev.step(10, dt)
            states.append(ev.get_state())
    a, b = states
    assert np.linalg.norm(b - a) / np.linalg.norm(a) <= 1e-12


def test_refusals():
    bricks = [Brick((2, 2, 2))]
    with pytest.raises(DgswError):
        DgEvolution(bricks, [4, 5, 4, 5, 4, 5, 4, 5], precision=PRECISION_DOUBLE_FLOAT)
    with pytest.raises(DgswError):
        DgEvolution(bricks, 4, precision=PRECISION_DOUBLE_FLOAT, time_stepper="adams_bashforth")
    with DgEvolution(bricks, 4, precision=PRECISION_DOUBLE_FLOAT) as ev:
        with pytest.raises(DgswError):
            ev.substep(0, 1e-3)
        with pytest.raises(DgswError):
            ev.set_exponential_filter(36.0, 32)
        ev.step(1, 1e-3)  # the handle stays usable


def test_misfit_gradient_matches_fp64():
    # a double-float handle runs the misfit forward and adjoint sweep on the
    # same Taylor kernels as the mixed-precision problem
    from spectre_gb300.adjoint import MisfitProblem
    kw = dict(elements=(4, 4, 4), points=6, dt=1e-3, steps=40, steps_per_window=10,
              n_samples=12, seed=5)
    pd = MisfitProblem(precision="fp64", **kw)
    try:
        psi0 = pd.initial_psi()
        J64, g64 = pd.value_and_gradient(psi0)
        with DgEvolution([Brick((4, 4, 4))], 6, precision=PRECISION_DOUBLE_FLOAT) as ev:
            ev.set_samples(pd.xyz)
            ev.set_state(pd._state(psi0))
            J = ev.misfit_forward(pd.targets, pd.steps_per_window, pd.dt)
            g = ev.misfit_adjoint().reshape(pd.n_elem, 5, -1)[:, 0, :].reshape(g64.shape)
        assert J == pytest.approx(J64, rel=1e-11)
        assert float((g - g64).abs().max()) <= 1e-10 * float(g64.abs().max())
    finally:
        pd.close()


def test_step_host_equals_device_steps():
    # the host-state call on a double-float handle: whole-state copies around
    # the same device steps, bit-identical to set_state + step + get_state
    bricks = [Brick((3, 3, 2))]
    n, dt = 6, 1e-3
    u = np.random.default_rng(3).uniform(-1, 1, 18 * 5 * n ** 3)
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        ev.set_state(u)
        ev.step(4, dt)
        ref = ev.get_state()
        got = ev.step_host(u.copy(), 4, dt)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("steps", [1, 2, 5])
def test_pipelined_step_host_equals_device_steps(steps):
    # 16^3 elements: enough for the chunked host-state path, whose copies
    # overlap the first and last steps' launches chunk by chunk; the same
    # bits as set_state + step + get_state
    import torch
    bricks = [Brick((16, 16, 16))]
    n, dt = 4, 1e-3
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        u = np.random.default_rng(steps).uniform(-1, 1, ev.state_size)
        ev.set_state(u)
        ev.step(steps, dt)
        ref = ev.get_state()
        host = torch.from_numpy(u.copy()).pin_memory()
        got = ev.step_host(host.numpy(), steps, dt)
    np.testing.assert_array_equal(got, ref)


def test_graph_chunks_equal_single_steps(oracle):
    # dgsw_step replays windows of steps from CUDA graphs: 37 steps (two
    # graphs of 16 and single steps) give the bits of 37 single calls
    bricks = [Brick((2, 2, 2))]
    n, dt = 6, 1e-3
    u0 = oracle.initial_data(bricks, n, "gaussian", oracle.gaussian_params(1, width=1.0))
    with DgEvolution(bricks, n, precision=PRECISION_DOUBLE_FLOAT) as ev:
        ev.set_state(u0)
        ev.step(37, dt)
        a = ev.get_state()
        ev.set_state(u0)
        for _ in range(37):
            ev.step(1, dt)
        b = ev.get_state()
    np.testing.assert_array_equal(a, b)
