"""Discrete adjoint of the FP64 DG step: transpose identities, the oracle's
assembled operator, central differences and a tangent-linear run.

Tolerances: transpose identities <= 1e-12 relative; gradients vs central
differences (eps = 1e-6; J is exactly quadratic in Psi0, so the difference
quotient has no truncation error) <= 1e-6 relative; adjoint vs
tangent-linear <= 1e-10 relative.
"""
import math

import numpy as np
import pytest

from spectre_gb300.adjoint import MisfitProblem, misfit_function, psi_view
from spectre_gb300.dgsw import Brick, DgEvolution

pytestmark = pytest.mark.gpu


def test_transpose_identity_config4_size():
    import torch
    with DgEvolution([Brick((8, 8, 8))], 8) as ev:
        g = torch.Generator(device="cuda").manual_seed(1)
        u = torch.rand(ev.state_size, dtype=torch.float64, device="cuda", generator=g) - 0.5
        v = torch.rand(ev.state_size, dtype=torch.float64, device="cuda", generator=g) - 0.5
        lu = ev.rhs(u)
        ltv = ev.adjoint_rhs(v)
        a = float(torch.dot(lu, v))
        b = float(torch.dot(u, ltv))
        scale = float(lu.abs().sum() * v.abs().max())
    assert abs(a - b) <= 1e-12 * scale, (a, b)


@pytest.mark.parametrize("n", [3, 4])
def test_adjoint_rhs_matches_oracle_transpose(oracle, n):
    import torch
    bricks = [Brick((2, 2, 1), (0.0, 0.0, 0.0), (1.0, 2.0, 1.5))]
    size = int(oracle.offsets(oracle.elem_points(bricks, n))[-1])
    # assemble the oracle's operator column by column
    Lm = np.zeros((size, size))
    e = np.zeros(size)
    for j in range(size):
        e[:] = 0.0
        e[j] = 1.0
        Lm[:, j] = oracle.rhs(bricks, n, e)
    rng = np.random.default_rng(n)
    v = rng.uniform(-1, 1, size)
    with DgEvolution(bricks, n) as ev:
        got = ev.adjoint_rhs(torch.tensor(v, device="cuda")).cpu().numpy()
    ref = Lm.T @ v
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def small_problem():
    return MisfitProblem(elements=(4, 4, 4), points=6, dt=1e-3, steps=60, steps_per_window=10,
                         n_samples=16, seed=9)


def test_gradient_vs_central_differences():
    import torch
    p = small_problem()
    try:
        psi0 = p.initial_psi()
        J, g = p.value_and_gradient(psi0)
        assert J > 0
        rng = torch.Generator(device="cuda").manual_seed(5)
        eps = 1e-6
        for _ in range(16):
            v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
            fd = (p.value(psi0 + eps * v) - p.value(psi0 - eps * v)) / (2 * eps)
            ad = float(torch.sum(g * v))
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30) + 1e-12, (fd, ad)
    finally:
        p.close()


def test_gradient_vs_tangent_linear():
    import torch
    p = small_problem()
    try:
        psi0 = p.initial_psi()
        J, g = p.value_and_gradient(psi0)
        rng = torch.Generator(device="cuda").manual_seed(6)
        for _ in range(3):
            v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
            tl = p.tangent_linear(psi0, v)
            ad = float(torch.sum(g * v))
            assert abs(tl - ad) <= 1e-10 * abs(tl), (tl, ad)
    finally:
        p.close()


def test_autograd_function():
    import torch
    p = small_problem()
    try:
        F = misfit_function()
        psi0 = p.initial_psi().requires_grad_(True)
        J = F.apply(psi0, p)
        J.backward()
        _, g = p.value_and_gradient(psi0.detach())
        # the sampler's adjoint adds with atomics: summation order (and so the
        # last bits) may differ between two sweeps
        scale = float(g.abs().max())
        assert float((psi0.grad - g).abs().max()) <= 1e-12 * scale
        assert float(J.detach()) == pytest.approx(p.value(psi0.detach()), rel=1e-13)
    finally:
        p.close()


@pytest.mark.slow
def test_config4_gradient_checks():
    # The adjoint case at full size: 8^3 elements x 8^3 points, dt 5e-4, 2000 steps,
    # 64 samples every 10 steps; 16 central-difference directions and one
    # tangent-linear direction
    import torch
    p = MisfitProblem()
    try:
        psi0 = p.initial_psi()
        J, g = p.value_and_gradient(psi0)
        rng = torch.Generator(device="cuda").manual_seed(7)
        eps = 1e-6
        worst = 0.0
        for _ in range(16):
            v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
            fd = (p.value(psi0 + eps * v) - p.value(psi0 - eps * v)) / (2 * eps)
            ad = float(torch.sum(g * v))
            worst = max(worst, abs(fd - ad) / abs(ad))
        assert worst <= 1e-6, worst
        v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
        tl = p.tangent_linear(psi0, v)
        assert abs(tl - float(torch.sum(g * v))) <= 1e-10 * abs(tl)
    finally:
        p.close()
