"""Exponential filter (Filters::Exponential applied by dg::Actions::Filter
after every substep).

CPU: the oracle's 1D filter matrix against the reference's known answer
(Test_Filtering.cpp: each Legendre mode k is damped by
exp(-alpha (k/(N-1))^(2 half_power)), 2e-12), and the product's host matrix
against the oracle's (1e-13).  GPU: filtered SSP-RK3 steps of the flat,
the mixed-extent and the curved paths against the oracle stepped substep by
substep with the filter (<= 1e-11 relative per variable); the same in mixed
precision (<= 1e-6), and the configuration-5 shell over 1000 filtered steps,
mixed against FP64 (rel L2 <= 1e-6).
"""
import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, CurvedDgEvolution, DgEvolution, Shell

ALPHA, HALF_POWER = 36.0, 8


@pytest.mark.parametrize("alpha", [10.0, 20.0, 30.0, 40.0])
@pytest.mark.parametrize("half_power", [2, 4, 8, 16])
def test_oracle_filter_damps_legendre_modes(oracle, alpha, half_power):
    for n in range(2, 21):
        F = oracle.exponential_filter(n, alpha, half_power)
        V = oracle.vandermonde(n)
        Vi = oracle.inv_vandermonde(n)
        for modal in (np.full(n, float(n)), np.arange(1.0, n + 1.0)):
            got = Vi @ (F @ (V @ modal))
            want = modal * np.exp(-alpha * (np.arange(n) / (n - 1.0)) ** (2 * half_power))
            assert np.all(np.abs(got - want) <= 2e-12 * (1.0 + np.abs(want))), n


@pytest.mark.parametrize("n", range(2, 13))
def test_product_filter_matrix_matches_oracle(dgsw_lib, oracle, n):
    for alpha, hp in ((12.0, 32), (36.0, 8), (0.0, 4)):
        np.testing.assert_allclose(dgsw.exponential_filter_matrix(n, alpha, hp),
                                   oracle.exponential_filter(n, alpha, hp), rtol=0, atol=1e-13)


@pytest.mark.parametrize("n", range(2, 13))
def test_filter_matrix_mirror_symmetry(dgsw_lib, n):
    # the filter kernels apply F through its mirror symmetry F[N-1-i][N-1-j]
    # = F[i][j] (symmetric LGL nodes, Legendre parity); the host matrices
    # hold it to rounding, and the even/odd form reproduces F x
    rng = np.random.default_rng(n)
    for alpha, hp in ((12.0, 32), (36.0, 8), (0.0, 4)):
        F = dgsw.exponential_filter_matrix(n, alpha, hp)
        np.testing.assert_allclose(F[::-1, ::-1], F, rtol=0, atol=1e-14)
        h = n // 2
        A = 0.5 * (F[:h, :h] + F[:h, ::-1][:, :h])
        B = 0.5 * (F[:h, :h] - F[:h, ::-1][:, :h])
        for x in rng.standard_normal((4, n)):
            e = x[:h] + x[::-1][:h]
            o = x[:h] - x[::-1][:h]
            P = A @ e + (F[:h, h] * x[h] if n % 2 else 0.0)
            Q = B @ o
            y = np.empty(n)
            y[:h] = P + Q
            y[n - h:] = (P - Q)[::-1]
            if n % 2:
                y[h] = 0.5 * (F[h, :h] + F[h, ::-1][:h]) @ e + F[h, h] * x[h]
            np.testing.assert_allclose(y, F @ x, rtol=0, atol=1e-13 * (1 + np.abs(x).sum()))


def _rel(a, b, elem_n):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    num = np.zeros(5)
    den = np.zeros(5)
    off = 0
    for n in elem_n:
        npt = int(n) ** 3
        for v in range(5):
            sl = slice(off + v * npt, off + (v + 1) * npt)
            num[v] = max(num[v], np.abs(a[sl] - b[sl]).max())
            den[v] = max(den[v], np.abs(b[sl]).max())
        off += 5 * npt
    return float(max(num[v] / den[v] if den[v] > 0 else num[v] for v in range(5)))


def _oracle_filtered(oracle, rhs, u, dt, steps, elem_n):
    u0 = np.array(u, dtype=np.float64).ravel()
    for _ in range(steps):
        cur = u0
        for k in range(3):
            cur = oracle.rk3_substep(k, dt, u0, cur, rhs(cur))
            cur = oracle.filter_elements(elem_n, cur, ALPHA, HALF_POWER)
        u0 = cur
    return u0


@pytest.mark.gpu
def test_flat_filtered_steps_match_oracle(oracle):
    bricks = [Brick((3, 2, 4))]
    n, dt = 7, 2e-3
    rng = np.random.default_rng(3)
    en = oracle.elem_points(bricks, n)
    u = rng.uniform(-1, 1, int(oracle.offsets(en)[-1]))
    ref = _oracle_filtered(oracle, lambda x: oracle.rhs(bricks, n, x), u, dt, 4, en)
    with DgEvolution(bricks, n) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u)
        ev.step(4, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-11
        # one substep at a time gives the same states
        ev.set_state(u)
        for _ in range(4):
            for k in range(3):
                ev.substep(k, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-11
        # switched off again: plain steps
        ev.set_exponential_filter(ALPHA, HALF_POWER, enable=False)
        ev.set_state(u)
        ev.step(1, dt)
        plain = oracle.evolve(bricks, n, u, dt, 1)
        assert _rel(ev.get_state(), plain, en) <= 1e-12


@pytest.mark.gpu
def test_mixed_extent_filtered_steps_match_oracle(oracle):
    bricks = [Brick((2, 3, 2))]
    rng = np.random.default_rng(5)
    pts = rng.integers(4, 11, size=12).astype(np.int32)
    dt = 1e-3
    en = oracle.elem_points(bricks, pts)
    u = rng.uniform(-1, 1, int(oracle.offsets(en)[-1]))
    ref = _oracle_filtered(oracle, lambda x: oracle.rhs(bricks, pts, x), u, dt, 3, en)
    with DgEvolution(bricks, pts) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u)
        ev.step(3, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-11


@pytest.mark.gpu
def test_curved_filtered_steps_match_oracle(oracle):
    n, dt = 6, 1e-2
    s = oracle.shell(1.9, 20.0, 1, 1, n, 1.0, 0.0, 1.0)
    u = oracle.shell_initial_data(s, 8.0, 1.0)
    E = u.shape[0]
    en = np.full(E, n, dtype=np.int32)
    rhs = lambda x: oracle.shell_rhs(s, x.reshape(u.shape))[0].ravel()  # noqa: E731
    ref = _oracle_filtered(oracle, rhs, u, dt, 5, en)
    with CurvedDgEvolution(Shell(1.9, 20.0, 1, 1), n, gamma2=1.0) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u.ravel())
        ev.step(5, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("n", [6, 7])
def test_mixed_filtered_steps_match_oracle(oracle, n):
    # mixed precision with the filter after every substep (filter_mixed.cu):
    # the residual (F - I) u0 in double-float, the filters of the increments
    # in FP32; against the oracle's FP64 filtered steps
    bricks = [Brick((3, 2, 4))]
    dt = 2e-3
    rng = np.random.default_rng(13 + n)
    en = oracle.elem_points(bricks, n)
    u = rng.uniform(-1, 1, int(oracle.offsets(en)[-1]))
    ref = _oracle_filtered(oracle, lambda x: oracle.rhs(bricks, n, x), u, dt, 4, en)
    with DgEvolution(bricks, n, precision=dgsw.PRECISION_MIXED) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u)
        ev.step(4, dt)
        a = ev.get_state()
        assert _rel(a, ref, en) <= 1e-6
        # one substep at a time gives the same states
        ev.set_state(u)
        for _ in range(4):
            for k in range(3):
                ev.substep(k, dt)
        np.testing.assert_array_equal(ev.get_state(), a)


@pytest.mark.gpu
def test_mixed_extent_mixed_filtered_steps_match_oracle(oracle):
    bricks = [Brick((2, 3, 2))]
    rng = np.random.default_rng(6)
    pts = rng.integers(4, 11, size=12).astype(np.int32)
    dt = 1e-3
    en = oracle.elem_points(bricks, pts)
    u = rng.uniform(-1, 1, int(oracle.offsets(en)[-1]))
    ref = _oracle_filtered(oracle, lambda x: oracle.rhs(bricks, pts, x, gamma2=0.5), u, dt, 3, en)
    with DgEvolution(bricks, pts, precision=dgsw.PRECISION_MIXED, gamma2=0.5) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u)
        ev.step(3, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-6


@pytest.mark.gpu
def test_curved_mixed_filtered_steps_match_oracle(oracle):
    n, dt = 6, 1e-2
    s = oracle.shell(1.9, 20.0, 1, 1, n, 1.0, 0.0, 1.0)
    u = oracle.shell_initial_data(s, 8.0, 1.0)
    E = u.shape[0]
    en = np.full(E, n, dtype=np.int32)
    rhs = lambda x: oracle.shell_rhs(s, x.reshape(u.shape))[0].ravel()  # noqa: E731
    ref = _oracle_filtered(oracle, rhs, u, dt, 5, en)
    with CurvedDgEvolution(Shell(1.9, 20.0, 1, 1), n, gamma2=1.0,
                           precision=dgsw.PRECISION_MIXED) as ev:
        ev.set_exponential_filter(ALPHA, HALF_POWER)
        ev.set_state(u.ravel())
        ev.step(5, dt)
        assert _rel(ev.get_state(), ref, en) <= 1e-6


@pytest.mark.gpu
@pytest.mark.slow
def test_curved_mixed_filtered_config5_full_run():
    # the configuration-5 shell (768 elements x 10^3 points, Kerr-Schild M = 1,
    # gamma1 = 0, gamma2 = 1, dt = 1e-3) over its 1000 steps with the filter
    # after every substep, as the reference's curved executable's step
    # actions apply it: mixed precision against FP64, rel L2 <= 1e-6
    states = []
    for prec in (dgsw.PRECISION_FP64, dgsw.PRECISION_MIXED):
        sh = Shell(1.9, 20.0, 2, 3, "logarithmic", 1.0, 0.0)
        with CurvedDgEvolution(sh, 10, precision=prec, gamma2=1.0) as ev:
            ev.set_exponential_filter(ALPHA, HALF_POWER)
            ev.set_gaussian_shell(1.0, 8.0, 1.0)
            ev.step(1000, 1e-3)
            states.append(ev.get_state())
    a, m = states
    assert np.isfinite(m).all()
    err = float(np.linalg.norm(m - a) / np.linalg.norm(a))
    print("curved mixed vs FP64, both filtered, 1000 steps: rel L2 %.3e" % err)
    assert err <= 1e-6
