"""Legendre-Gauss quadrature (Spectral::Quadrature::Gauss) for the flat
scalar wave: faces interpolated with boundary_interpolation_matrices and
corrections lifted into the element by lift_boundary_terms_gauss_points.

CPU: the oracle's nodes, weights and D against the reference's decimals
(Test_LegendreGauss.cpp, 1e-14); the reference's property checks of the
boundary interpolation and lifting terms (Test_Spectral.cpp:477-530);
the product's host tables against the oracle (1e-14); spectral convergence
of the oracle's Gauss right-hand side and of its evolution to the plane wave.
GPU: the Gauss right-hand side and steps against the oracle (<= 1e-12
relative per variable), with and without gamma2.
"""
import json
import math
import os

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, DgEvolution

HERE = os.path.dirname(os.path.abspath(__file__))
GG = json.load(open(os.path.join(HERE, "golden", "gauss_golden.json")))


@pytest.mark.parametrize("n", sorted(int(k) for k in GG["points_weights"]))
def test_oracle_gauss_points_weights_and_D_golden(oracle, n):
    x, w = oracle.lg(n)
    g = GG["points_weights"][str(n)]
    # the reference's decimals carry 15 digits
    np.testing.assert_allclose(x, g["x"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(w, g["w"], rtol=0, atol=2e-15)
    np.testing.assert_allclose(oracle.lg_diff_matrix(n), np.array(GG["diff_matrix"][str(n)]),
                               rtol=0, atol=2e-14)


@pytest.mark.parametrize("n", range(2, 21))
def test_oracle_gauss_boundary_terms_properties(oracle, n):
    x, w = oracle.lg(n)
    lo, hi, llo, lhi = oracle.lg_boundary(n)
    for p in range(n):
        u = x ** p
        assert abs(lo @ u - (-1.0) ** p) < 1e-12
        assert abs(hi @ u - 1.0) < 1e-12
    np.testing.assert_allclose(llo, lo / w, rtol=1e-15)
    np.testing.assert_allclose(lhi, hi / w, rtol=1e-15)
    # the Gauss rule integrates degree 2n - 1 exactly
    assert abs(w @ x ** (2 * n - 2) - 2.0 / (2 * n - 1)) < 1e-13


@pytest.mark.parametrize("n", range(2, 13))
def test_product_gauss_tables_match_oracle(dgsw_lib, oracle, n):
    g = dgsw.gauss_spectral(n)
    x, w = oracle.lg(n)
    lo, hi, llo, lhi = oracle.lg_boundary(n)
    np.testing.assert_allclose(g["x"], x, rtol=0, atol=1e-15)
    np.testing.assert_allclose(g["w"], w, rtol=1e-14)
    np.testing.assert_allclose(g["D"], oracle.lg_diff_matrix(n), rtol=0, atol=1e-12)
    for a, b in ((g["interp_lower"], lo), (g["interp_upper"], hi), (g["lift_lower"], llo),
                 (g["lift_upper"], lhi)):
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-14)


def test_oracle_gauss_rhs_and_evolution_converge(oracle):
    b = [Brick((2, 2, 2))]
    errs, evo = [], []
    for n in (4, 6, 8, 10):
        u = oracle.plane_wave_gauss(b, n, [1, 1, 1])
        du = oracle.rhs_gauss(b, n, u)
        ph = oracle.coords_gauss(b, n).sum(1)
        om = math.sqrt(3.0)
        ex = np.zeros_like(u)
        ex[:, 0] = -om * np.cos(ph)
        ex[:, 1] = 3.0 * np.sin(ph)
        ex[:, 2:] = (om * np.sin(ph))[:, None]
        errs.append(np.abs(du - ex).max())
        if n <= 8:
            u1 = oracle.evolve_gauss(b, n, u, 1e-3, 50)
            evo.append(np.abs(u1 - oracle.plane_wave_gauss(b, n, [1, 1, 1], t=0.05)).max())
    assert all(a > 10 * c for a, c in zip(errs, errs[1:])), errs
    assert all(a > 10 * c for a, c in zip(evo, evo[1:])), evo
    assert errs[-1] < 1e-4


def _rel(a, b, n):
    a = np.asarray(a).reshape(-1, 5, n ** 3)
    b = np.asarray(b).reshape(-1, 5, n ** 3)
    return max(np.abs(a[:, v] - b[:, v]).max() / np.abs(b[:, v]).max() for v in range(5))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_gpu_gauss_rhs_matches_oracle(oracle, n):
    bricks = [Brick((3, 2, 2))]
    rng = np.random.default_rng(40 + n)
    E = 12
    u = rng.uniform(-1, 1, E * 5 * n ** 3)
    for g2 in (0.0, 1.5):
        with DgEvolution(bricks, n, gamma2=g2, quadrature="gauss") as ev:
            got = ev.rhs(u)
        assert _rel(got, oracle.rhs_gauss(bricks, n, u, gamma2=g2), n) <= 1e-12


@pytest.mark.gpu
def test_gpu_gauss_steps_match_oracle(oracle):
    bricks = [Brick((4, 4, 4))]
    n, dt = 6, 1e-3
    u = oracle.plane_wave_gauss(bricks, n, [1, 1, 1]).ravel()
    ref = oracle.evolve_gauss(bricks, n, u, dt, 20)
    with DgEvolution(bricks, n, quadrature="gauss") as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        np.testing.assert_allclose(ev.get_state(), u, rtol=0, atol=1e-14)
        ev.step(20, dt)
        assert _rel(ev.get_state(), ref, n) <= 1e-11
        ev.set_state(u)
        for _ in range(20):
            for k in range(3):
                ev.substep(k, dt)
        assert _rel(ev.get_state(), ref, n) <= 1e-11
        err = ev.observe_plane_wave_errors([1.0, 1.0, 1.0], 20 * dt)
        assert err["L2Norm(Error(Psi))"] < 5e-3


@pytest.mark.gpu
def test_gpu_gauss_unsupported_combinations():
    with pytest.raises(dgsw.DgswError):
        DgEvolution([Brick((2, 2, 2))], 6, precision=dgsw.PRECISION_MIXED, quadrature="gauss")
    with DgEvolution([Brick((2, 2, 2))], 6, quadrature="gauss") as ev:
        with pytest.raises(dgsw.DgswError):
            ev.set_exponential_filter(12.0, 32)
