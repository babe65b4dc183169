"""StepChoosers::Cfl per element (dgsw_cfl_steps, host-only) and the stable
steps it uses, checked the way the reference's TimeStepperTestUtils
stability_test checks stable_step (TimeStepperTestUtils.cpp:266-333)."""
import math

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, Shell


def _stable_step(time_stepper, order=3):
    # back out stable_step from the Cfl step of a unit-speed affine element
    n, L = 6, 2.0
    x, _ = dgsw.lgl_points_weights(n)
    spacing = 0.5 * L * (x[1] - x[0])
    step = dgsw.cfl_steps([Brick((1, 1, 1), (0, 0, 0), (L, L, L))], n, 1.0,
                          time_stepper=time_stepper, order=order)[0]
    return step * 3.0 / spacing


def _spectral_radius(stepper, h, lam):
    """Largest |eigenvalue| of the step operator of y' = lam y."""
    if stepper == "rk3":
        # Rk3HesthavenSsp: u1 = u + h f(u); u2 = 3/4 u + 1/4 (u1 + h f(u1));
        # u3 = 1/3 u + 2/3 (u2 + h f(u2))
        z = h * lam
        u1 = 1 + z
        u2 = 0.75 + 0.25 * (u1 + z * u1)
        return abs(1 / 3 + 2 / 3 * (u2 + z * u2))
    k = stepper
    c = dgsw.adams_coefficients(list(range(k)), k - 1, k)  # oldest first, unit step
    # companion matrix on (f_{n-k+1} ... f_n, y_n) for f = lam y
    A = np.zeros((k, k), dtype=complex)
    for i in range(k - 1):
        A[i, i + 1] = 1.0
    # y_{n+1} = y_n + h sum_j c_j lam y_{n-k+1+j}
    A[k - 1, :] = h * lam * c
    A[k - 1, k - 1] += 1.0
    return max(abs(np.linalg.eigvals(A)))


@pytest.mark.parametrize("stepper", ["rk3", 1, 2, 3, 4, 5, 6, 7, 8])
def test_stable_steps_bracket_the_stability_limit(stepper):
    # y' = (exp(i pi) - 1) y: stable just below stable_step, unstable above
    # (stability_test with bracket 1.001)
    if stepper == "rk3":
        s = _stable_step("rk3_hesthaven_ssp")
    else:
        s = _stable_step("adams_bashforth", stepper)
    lam = complex(math.cos(math.pi), math.sin(math.pi)) - 1.0
    assert _spectral_radius(stepper, s / 1.001, lam) <= 1.0 + 1e-12
    assert _spectral_radius(stepper, s * 1.001, lam) > 1.0


def test_cfl_affine_elements():
    b = [Brick((3, 2, 4), (0.0, 0.0, 0.0), (1.5, 1.0, 2.0))]
    n = 7
    steps = dgsw.cfl_steps(b, n, 0.5)
    x, _ = dgsw.lgl_points_weights(n)
    r = np.cbrt(4 + np.sqrt(17))
    stable = 0.5 * (1 + r - 1 / r)
    width = min(1.5 / 3, 1.0 / 2, 2.0 / 4)
    want = 0.5 * stable * 0.5 * width * (x[1] - x[0]) / 3
    assert steps.shape == (24,)
    np.testing.assert_allclose(steps, want, rtol=1e-14)


def test_cfl_shell_matches_restatement():
    # minimum_grid_spacing over neighbours one index away
    # (Domain/MinimumGridSpacing.cpp) and CurvedScalarWave's largest speed
    # max(|1 + gamma1| |beta|, |beta| + alpha) on Kerr-Schild
    shell = Shell(1.9, 20.0, 0, 1, "logarithmic", 1.0, 0.3)
    n = 5
    steps = dgsw.cfl_steps(shell, n, 1.0)
    xyz, _, _ = dgsw.shell_geometry(shell, n)
    E = xyz.shape[0]
    r3 = np.cbrt(4 + np.sqrt(17))
    stable = 0.5 * (1 + r3 - 1 / r3)
    for e in range(E):
        X = xyz[e].reshape(3, n, n, n)  # [c][k][j][i]
        P = np.moveaxis(X, 0, -1)
        best = np.inf
        for dk in (-1, 0, 1):
            for dj in (-1, 0, 1):
                for di in (-1, 0, 1):
                    if (dk, dj, di) == (0, 0, 0):
                        continue
                    a = P[max(0, -dk):n - max(0, dk), max(0, -dj):n - max(0, dj),
                          max(0, -di):n - max(0, di)]
                    b = P[max(0, dk):n - max(0, -dk), max(0, dj):n - max(0, -dj),
                          max(0, di):n - max(0, -di)]
                    best = min(best, np.sqrt(((a - b) ** 2).sum(-1)).min())
        r = np.sqrt((P ** 2).sum(-1))
        H = 1.0 / r
        alpha = 1 / np.sqrt(1 + 2 * H)
        beta = 2 * H * alpha
        speed = np.maximum(1.3 * beta, beta + alpha).max()
        assert steps[e] == pytest.approx(stable * best / (3 * speed), rel=1e-12)


def test_levels_from_cfl():
    s = np.array([1.0, 0.5, 0.26, 0.125, 0.9])
    np.testing.assert_array_equal(dgsw.levels_from_cfl(s, 1.0), [0, 1, 2, 3, 1])
    with pytest.raises(ValueError):
        dgsw.levels_from_cfl([0.01], 1.0)
