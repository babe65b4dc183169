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


@pytest.mark.parametrize("n", [4, 5, 8])
def test_mixed_gamma2_rhs_matches_oracle(oracle, n):
    # gamma2 (d_i Psi - Phi_i) in the time derivative and -gamma2 Psi in the
    # upwind characteristic field (TimeDerivative.cpp:37-44, UpwindPenalty.cpp:35-108)
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (1.0, 1.5, 2.0))]
    rng = np.random.default_rng(10 + n)
    u = oracle.initial_data(bricks, n, "gaussian", oracle.gaussian_params(1, width=0.7,
                                                                         center=(0.4, 0.8, 1.1)))
    u += 0.1 * rng.uniform(-1, 1, u.size)
    ref = oracle.rhs(bricks, n, u, gamma2=1.5)
    with DgEvolution(bricks, n, precision=PRECISION_MIXED, gamma2=1.5) as ev:
        got = ev.rhs(u)
    E = len(u) // (5 * n ** 3)
    a = got.reshape(E, 5, -1)
    b = ref.reshape(E, 5, -1)
    per_var = [np.max(np.abs(a[:, v] - b[:, v])) / np.max(np.abs(b[:, v])) for v in range(5)]
    assert max(per_var) <= 1e-6, per_var


@pytest.mark.parametrize("gamma2", [0.7, 1.5])
def test_mixed_gamma2_evolution_matches_oracle(oracle, gamma2):
    # the config-1 grid (4^3 x 6^3 plane wave, dt 1e-3) for 200 steps with
    # constraint damping; the plane wave satisfies Phi = grad Psi, so perturb
    # Phi to exercise the damping term
    bricks = [Brick((4, 4, 4))]
    n, dt, steps = 6, 1e-3, 200
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    E = len(u0) // (5 * n ** 3)
    v = u0.reshape(E, 5, -1).copy()
    v[:, 2:] *= 1.05
    u0 = v.ravel()
    with DgEvolution(bricks, n, precision=PRECISION_MIXED, gamma2=gamma2) as ev:
        ev.set_state(u0)
        ev.step(steps, dt)
        got = ev.get_state()
        # substeps one at a time against update_u as well
        ev.set_state(u0)
        cur = u0
        for k in range(3):
            sub = oracle.rk3_substep(k, dt, u0, cur, oracle.rhs(bricks, n, cur, gamma2=gamma2))
            ev.substep(k, dt)
            assert rel_linf(ev.get_state(), sub) <= 1e-9, k
            cur = sub
    ref = oracle.evolve(bricks, n, u0, dt, steps, gamma2=gamma2)
    assert rel_l2(got, ref) <= 1e-6


def test_mixed_gamma2_differing_extents_matches_oracle(oracle):
    from spectre_gb300 import workloads
    bricks, pts, params = workloads.batched_instances(6, seed=31)
    dt, steps = 1e-4, 40
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    with DgEvolution(bricks, pts, precision=PRECISION_MIXED, gamma2=1.5) as ev:
        ev.set_state(u0)
        ev.step(steps, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, pts, u0, dt, steps, gamma2=1.5)
    off = 0
    e = 0
    for b in bricks:
        ne = b.elements[0] * b.elements[1] * b.elements[2]
        size = int(5 * np.sum(np.asarray(pts[e:e + ne], dtype=np.int64) ** 3))
        assert rel_l2(got[off:off + size], ref[off:off + size]) <= 1e-6
        off += size
        e += ne


@pytest.mark.parametrize("n", [6, 8])
def test_mixed_pipe_launch_shapes_agree(oracle, n):
    # the pipelined kernel's four candidates (dgsw_tune: one or two pipeline
    # buffers, the FP64 update as a separate stream or in the last stage's
    # epilogue): same bits, and all within the mixed bar of the FP64 oracle
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
        assert len(info["ms_per_step"]) == 4
        assert all(ms > 0 for ms in info["ms_per_step"])
        for v in range(len(info["ms_per_step"])):
            assert ev.tune(force_variant=v)["variant"] == v
            ev.set_state(u0)
            ev.step(steps, dt)
            out.append(ev.get_state())
    for got in out:
        assert rel_l2(got, ref) <= 1e-6
    for got in out[1:]:
        np.testing.assert_array_equal(out[0], got)
