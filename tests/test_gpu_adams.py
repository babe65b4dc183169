"""AdamsBashforth with local time stepping: the CUDA path through the C ABI
against the oracle's literal per-element, per-mortar evolution
(oracle/adams_oracle.cpp).

Tolerance: FP64 path, 1e-12 relative per step (max over variables of the
max-norm of the difference over the oracle's max-norm), accumulated over the
run's steps at the finest level, self-start steps included.  The product
integrates the variable-step Lagrange weights by Gauss-Legendre quadrature
where the reference expands them in monomials, so the weights differ in the
last bits; with the large, cancelling weights of high-order self-start
histories the state differs by up to ~1e-13 per step.
"""
import math

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick, DgEvolution

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def tol(order, slabs, L=0):
    """1e-12 per step: self-start steps plus the finest level's steps."""
    return RTOL * (order * (order - 1) // 2 + slabs * 2 ** L)


def per_var_rel(a, b, E, n):
    a = a.reshape(E, 5, n ** 3)
    b = b.reshape(E, 5, n ** 3)
    return max(float(np.abs(a[:, v] - b[:, v]).max() / np.abs(b[:, v]).max()) for v in range(5))


def pattern(E, L, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, L + 1, size=E).astype(np.int32)


def gaussian_state(oracle, bricks, n):
    return oracle.initial_data(bricks, n, "gaussian",
                               oracle.gaussian_params(len(bricks), width=0.9,
                                                      center=(1.1, 0.7, 0.9)))


def run_gpu(bricks, n, u0, slab, slabs, order, levels, gamma2, calls=None):
    with DgEvolution(bricks, n, gamma2=gamma2, time_stepper="adams_bashforth", order=order,
                     step_levels=levels) as ev:
        ev.set_state(u0)
        for k in (calls or [slabs]):
            ev.step(k, slab)
        return ev.get_state(), ev.adams_info()


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_global_stepping_matches_oracle(oracle, order):
    n, gamma2 = 5, 0.6
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (2.0, 1.5, 1.5))]
    u0 = gaussian_state(oracle, bricks, n)
    slab, slabs = 0.01, 4
    got, info = run_gpu(bricks, n, u0, slab, slabs, order, None, gamma2)
    want = oracle.evolve_adams(bricks, n, u0, slab, slabs, order, gamma2=gamma2)
    E = oracle.num_elements(bricks)
    assert per_var_rel(got, want, E, n) <= tol(order, slabs)
    assert info["launches_per_slab"] == 1


def test_global_stepping_order_8(oracle):
    # The self-start weights of order 8 are badly conditioned (sum |c| is
    # ~2e4 times |sum c|); the reference's monomial integration of the
    # Lagrange basis (AdamsCoefficients.cpp:73-117), restated by the oracle,
    # carries ~5e-13 relative error in them, the product's quadrature ~2e-15
    # (tests/test_adams_schedule.py checks both against exact rationals), so
    # the two states agree to the conditioning times the oracle's error.
    n = 5
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (2.0, 1.5, 1.5))]
    u0 = gaussian_state(oracle, bricks, n)
    got, _ = run_gpu(bricks, n, u0, 0.01, 4, 8, None, 0.6)
    want = oracle.evolve_adams(bricks, n, u0, 0.01, 4, 8, gamma2=0.6)
    assert per_var_rel(got, want, oracle.num_elements(bricks), n) <= 1e-8


@pytest.mark.parametrize("L,order", [(1, 2), (1, 3), (2, 3), (2, 4), (3, 2), (3, 3)])
def test_local_stepping_matches_oracle(oracle, L, order):
    n, gamma2 = 4, 0.4
    bricks = [Brick((4, 3, 2), (0.0, 0.0, 0.0), (2.0, 1.5, 1.0))]
    E = oracle.num_elements(bricks)
    levels = pattern(E, L, seed=10 * L + order)
    levels[0] = L
    u0 = gaussian_state(oracle, bricks, n)
    slab, slabs = 0.02, 3
    got, info = run_gpu(bricks, n, u0, slab, slabs, order, levels, gamma2)
    want = oracle.evolve_adams(bricks, n, u0, slab, slabs, order, levels=levels, gamma2=gamma2)
    assert per_var_rel(got, want, E, n) <= tol(order, slabs, L)
    assert info["launches_per_slab"] == 2 ** L
    steps = sum(2 ** int(l) for l in levels)
    assert info["rhs_points_per_slab"] == steps * n ** 3


@pytest.mark.parametrize("n", [2, 3, 6, 7, 8, 9, 10, 11, 12])
def test_extents(oracle, n):
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2.0, 2.0, 2.0))]
    E = oracle.num_elements(bricks)
    levels = np.array([0, 1, 1, 0, 1, 0, 0, 1], np.int32)
    u0 = gaussian_state(oracle, bricks, n)
    got, _ = run_gpu(bricks, n, u0, 0.004, 2, 3, levels, 0.0)
    want = oracle.evolve_adams(bricks, n, u0, 0.004, 2, 3, levels=levels)
    assert per_var_rel(got, want, E, n) <= tol(3, 2, 1)


def test_slabs_continue_across_calls_and_restart_on_new_state(oracle):
    n = 4
    bricks = [Brick((2, 2, 3), (0.0, 0.0, 0.0), (1.0, 1.0, 1.5))]
    E = oracle.num_elements(bricks)
    levels = pattern(E, 2, seed=3)
    u0 = gaussian_state(oracle, bricks, n)
    want = oracle.evolve_adams(bricks, n, u0, 0.01, 5, 3, levels=levels)
    got, _ = run_gpu(bricks, n, u0, 0.01, 5, 3, levels, 0.0, calls=[2, 1, 2])
    assert per_var_rel(got, want, E, n) <= tol(3, 5, 2)
    with DgEvolution(bricks, n, time_stepper="adams_bashforth", order=3,
                     step_levels=levels) as ev:
        ev.set_state(np.zeros_like(u0))
        ev.step(2, 0.01)
        ev.set_state(u0)  # new initial values: self-start again
        ev.step(5, 0.01)
        assert per_var_rel(ev.get_state(), want, E, n) <= tol(3, 5, 2)


def test_uniform_level_equals_half_slab(oracle):
    # size-independent: every element on level 1 with slab 2 dt steps exactly
    # as every element on level 0 with slab dt
    n = 8
    bricks = [Brick((12, 12, 12), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    with DgEvolution(bricks, n, time_stepper="adams_bashforth", order=4,
                     step_levels=np.ones(12 ** 3, np.int32)) as a, \
            DgEvolution(bricks, n, time_stepper="adams_bashforth", order=4) as b:
        a.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        b.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        a.step(3, 0.004)
        b.step(6, 0.002)
        ua, ub = a.get_state(), b.get_state()
    assert float(np.abs(ua - ub).max()) <= tol(4, 6) * float(np.abs(ub).max())


def test_local_stepping_accuracy_large(oracle):
    # size-independent: a 24^3-element brick with random levels 0..2 agrees
    # with the parity-tested SSP-RK3 path at a small step to the size of
    # AB3's time error (the coarsest step, 0.002, is inside AB3's stability
    # limit for N = 6 elements of width 2 pi / 24)
    n = 6
    bricks = [Brick((24, 24, 24), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    levels = pattern(24 ** 3, 2, seed=5)
    with DgEvolution(bricks, n, time_stepper="adams_bashforth", order=3,
                     step_levels=levels) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        ev.step(100, 0.002)
        u_lts = ev.get_state()
    with DgEvolution(bricks, n) as rk:
        rk.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        rk.step(400, 0.0005)
        u_rk = rk.get_state()
    assert float(np.abs(u_lts - u_rk).max()) < 1e-6


@pytest.mark.parametrize("order,L", [(1, 0), (3, 0), (4, 0), (2, 1), (3, 2)])
def test_curved_shell_matches_oracle(oracle, order, L):
    # the reference's curved executable steps with AdamsBashforth (LTS):
    # Kerr-Schild shell, curved UpwindPenalty across wedges, radiation
    # condition on the outer sphere, gamma2 = 1
    from spectre_gb300.dgsw import CurvedDgEvolution, Shell
    n = 6
    s = oracle.shell(1.9, 20.0, 1, 1, n, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5)
    levels = pattern(E, L, seed=order) if L else None
    slab, slabs = 0.02, 3
    with CurvedDgEvolution(Shell(1.9, 20.0, 1, 1), n, gamma2=1.0, time_stepper="adams_bashforth",
                           order=order, step_levels=levels) as ev:
        ev.set_state(u0.ravel())
        ev.step(slabs, slab)
        got = ev.get_state()
    want = oracle.shell_evolve_adams(s, u0, slab, slabs, order, levels=levels).ravel()
    assert per_var_rel(got, want, E, n) <= tol(order, slabs, L)


def per_var_rel_extents(a, b, elem_n):
    """per_var_rel on the layout of per-element extents."""
    num, den = np.zeros(5), np.zeros(5)
    off = 0
    for n in elem_n:
        npt = int(n) ** 3
        for v in range(5):
            sl = slice(off + v * npt, off + (v + 1) * npt)
            num[v] = max(num[v], np.abs(a[sl] - b[sl]).max())
            den[v] = max(den[v], np.abs(b[sl]).max())
        off += 5 * npt
    return float(max(num[v] / den[v] for v in range(5)))


@pytest.mark.parametrize("order,L,gamma2", [(1, 0, 0.0), (3, 0, 0.6), (2, 1, 0.0), (3, 1, 0.6),
                                            (4, 2, 0.0), (3, 3, 0.0)])
def test_local_stepping_differing_extents_matches_oracle(oracle, order, L, gamma2):
    # p-nonconforming faces (extents 3..9 per element, mortars at the larger
    # extent) with step ratios up to 2^L against the oracle's literal
    # per-mortar, per-record-pair evolution
    bricks = [Brick((3, 3, 2), (0.0, 0.0, 0.0), (2.0, 2.0, 1.5)),
              Brick((2, 2, 2), (0.0, 0.0, 0.0), (1.5, 1.5, 1.5))]
    E = oracle.num_elements(bricks)
    rng = np.random.default_rng(100 * order + L)
    elem_n = rng.integers(3, 10, size=E).astype(np.int32)
    levels = pattern(E, L, seed=order + 7) if L else None
    u0 = oracle.initial_data(bricks, elem_n, "gaussian",
                             oracle.gaussian_params(len(bricks), width=0.7,
                                                    center=(0.9, 0.8, 0.7)))
    slab, slabs = 0.004, 3
    with DgEvolution(bricks, elem_n, gamma2=gamma2, time_stepper="adams_bashforth", order=order,
                     step_levels=levels) as ev:
        ev.set_state(u0)
        ev.step(slabs, slab)
        got = ev.get_state()
        info = ev.adams_info()
    want = oracle.evolve_adams_extents(bricks, elem_n, u0, slab, slabs, order, levels=levels,
                                       gamma2=gamma2)
    assert per_var_rel_extents(got, want, elem_n) <= tol(order, slabs, L)
    lv = np.zeros(E, np.int64) if levels is None else levels.astype(np.int64)
    assert info["rhs_points_per_slab"] == int(np.sum(2 ** lv * elem_n.astype(np.int64) ** 3))


def test_local_stepping_differing_extents_converges(oracle):
    # the product's LTS run on a p-nonconforming mesh against a time-resolved
    # SSP-RK3 run of the same semi-discrete system: AB3 error shrinks at
    # third order with the slab
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    elem_n = np.array([4, 5, 6, 4, 5, 4, 6, 5], np.int32)
    levels = np.array([0, 1, 0, 1, 1, 0, 1, 0], np.int32)
    T = 0.4
    u0 = oracle.initial_data(bricks, elem_n, "plane_wave", [1.0, 1.0, 1.0])
    with DgEvolution(bricks, elem_n) as rk:
        rk.set_state(u0)
        rk.step(800, T / 800)
        ref = rk.get_state()
    errs = []
    for s in (8, 16):
        with DgEvolution(bricks, elem_n, time_stepper="adams_bashforth", order=3,
                         step_levels=levels) as ev:
            ev.set_state(u0)
            ev.step(s, T / s)
            errs.append(float(np.abs(ev.get_state() - ref).max()))
    assert math.log2(errs[0] / errs[1]) > 2.5


@pytest.mark.parametrize("order,L", [(1, 0), (3, 0), (2, 1), (3, 2)])
def test_curved_shell_filtered_matches_oracle(oracle, order, L):
    # the curved executable's step actions in full: AdamsBashforth with local
    # time stepping and dg::Actions::Filter (Exponential, alpha 36, half
    # power 8) on every element after each of its steps, self-start included
    from spectre_gb300.dgsw import CurvedDgEvolution, Shell
    n = 6
    s = oracle.shell(1.9, 20.0, 1, 1, n, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5)
    levels = pattern(E, L, seed=order + 3) if L else None
    slab, slabs = 0.02, 3
    with CurvedDgEvolution(Shell(1.9, 20.0, 1, 1), n, gamma2=1.0, time_stepper="adams_bashforth",
                           order=order, step_levels=levels) as ev:
        ev.set_exponential_filter(36.0, 8)
        ev.set_state(u0.ravel())
        ev.step(slabs, slab)
        got = ev.get_state()
    want = oracle.shell_evolve_adams(s, u0, slab, slabs, order, levels=levels,
                                     filter=(36.0, 8)).ravel()
    assert per_var_rel(got, want, E, n) <= tol(order, slabs, L)


def test_flat_adams_refuses_the_filter(oracle):
    # the flat 3D scalar-wave executable does not filter; the flat LTS path
    # says so rather than stepping unfiltered
    from spectre_gb300.dgsw import DgswError
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2.0, 2.0, 2.0))]
    with DgEvolution(bricks, 4, time_stepper="adams_bashforth", order=2) as ev:
        ev.set_exponential_filter(36.0, 8)
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        with pytest.raises(DgswError):
            ev.step(1, 0.01)


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("order,L,filt,n", [(1, 0, False, 6), (3, 0, False, 6), (2, 1, False, 6),
                                            (3, 2, False, 6), (3, 2, True, 6), (3, 1, True, 5),
                                            (2, 1, False, 7)])
def test_curved_shell_mixed_adams_close_to_fp64(oracle, order, L, filt, n):
    # AdamsBashforth with local time stepping in mixed precision: each record
    # dt u = L(u) by the compensated double-float stage (FP32 result), the
    # FP64 state and the FP64 state records for the face coupling; against
    # the FP64 run of the same schedule (filtered or not) over 40 slabs
    from spectre_gb300.dgsw import CurvedDgEvolution, Shell, PRECISION_FP64, PRECISION_MIXED
    s = oracle.shell(1.9, 20.0, 1, 1, n, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5).ravel()
    levels = pattern(E, L, seed=order + 11) if L else None
    out = {}
    for prec in (PRECISION_FP64, PRECISION_MIXED):
        with CurvedDgEvolution(Shell(1.9, 20.0, 1, 1), n, precision=prec, gamma2=1.0,
                               time_stepper="adams_bashforth", order=order,
                               step_levels=levels) as ev:
            if filt:
                ev.set_exponential_filter(36.0, 8)
            ev.set_state(u0)
            ev.step(40, 0.02)
            out[prec] = ev.get_state()
    assert np.isfinite(out[PRECISION_MIXED]).all()
    assert rel_l2(out[PRECISION_MIXED], out[PRECISION_FP64]) <= 1e-6
