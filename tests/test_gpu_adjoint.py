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


@pytest.mark.parametrize("n", [3, 8, 10])
def test_adjoint_work_splits_agree(oracle, n):
    # both work splits of the adjoint kernel (N^2 threads per element with the
    # axes in turn; 3 N^2 with the axes at once) give the same bits, and at
    # n = 3 the oracle's assembled transpose
    import torch
    bricks = [Brick((3, 2, 2), (0.0, 0.0, 0.0), (1.0, 2.0, 1.5))]
    with DgEvolution(bricks, n) as ev:
        g = torch.Generator(device="cuda").manual_seed(n)
        v = torch.rand(ev.state_size, dtype=torch.float64, device="cuda", generator=g) - 0.5
        outs = []
        for split in (0, 1):
            chosen, ms = ev.adjoint_autotune(split)
            assert chosen == split and (ms > 0).all()
            outs.append(ev.adjoint_rhs(v))
        assert torch.equal(outs[0], outs[1])
        if n == 3:
            size = ev.state_size
            Lm = np.zeros((size, size))
            e = np.zeros(size)
            for j in range(size):
                e[:] = 0.0
                e[j] = 1.0
                Lm[:, j] = oracle.rhs(bricks, n, e)
            ref = Lm.T @ v.cpu().numpy()
            got = outs[1].cpu().numpy()
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_adjoint_gradient_same_bits_either_split():
    # the whole reverse sweep under each split: the same gradient (the
    # sampler's scatter adds with atomics, so compare to round-off)
    p = small_problem()
    try:
        psi0 = p.initial_psi()
        grads = []
        for split in (0, 1):
            p.ev.adjoint_autotune(split)
            grads.append(p.value_and_gradient(psi0)[1])
        scale = float(grads[0].abs().max())
        assert float((grads[0] - grads[1]).abs().max()) <= 1e-12 * scale
    finally:
        p.close()


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


# ---- mixed precision: FP64 states, double-float increments ---------------------
# Both sweeps run the step's Taylor polynomial with increments kept as (hi, lo)
# FP32 pairs (~44 bits), so the mixed objective and gradient follow the FP64
# ones to round-off: J <= 1e-11 relative and the gradient <= 1e-10 relative
# (max norm over the field; 2000 steps of the 8^3 x 8^3 case measured 2e-13
# and 4e-13).  Against central differences of the FP64 objective <= 1e-6
# relative, the bar of the FP64 gradient.

def _mixed_and_fp64(**kw):
    return MisfitProblem(precision="mixed", **kw), MisfitProblem(precision="fp64", **kw)


@pytest.mark.parametrize("elements,points", [((4, 4, 4), 6), ((3, 3, 3), 5), ((4, 4, 4), 8)])
def test_mixed_gradient_close_to_fp64(elements, points):
    kw = dict(elements=elements, points=points, dt=1e-3, steps=60, steps_per_window=10,
              n_samples=16, seed=9)
    pm, pd = _mixed_and_fp64(**kw)
    try:
        psi0 = pd.initial_psi()
        J64, g64 = pd.value_and_gradient(psi0)
        J32, g32 = pm.value_and_gradient(psi0)
        assert J32 == pytest.approx(J64, rel=1e-11)
        err = float((g32 - g64).abs().max()) / float(g64.abs().max())
        assert err <= 1e-10, err
    finally:
        pm.close()
        pd.close()


def test_mixed_gradient_vs_central_differences():
    import torch
    kw = dict(elements=(4, 4, 4), points=6, dt=1e-3, steps=60, steps_per_window=10,
              n_samples=16, seed=9)
    pm, pd = _mixed_and_fp64(**kw)
    try:
        psi0 = pd.initial_psi()
        _, g = pm.value_and_gradient(psi0)
        rng = torch.Generator(device="cuda").manual_seed(15)
        eps = 1e-6
        for _ in range(8):
            v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
            fd = (pd.value(psi0 + eps * v) - pd.value(psi0 - eps * v)) / (2 * eps)
            ad = float(torch.sum(g * v))
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30) + 1e-12, (fd, ad)
    finally:
        pm.close()
        pd.close()


def test_mixed_autograd_function():
    kw = dict(elements=(4, 4, 4), points=6, dt=1e-3, steps=30, steps_per_window=10,
              n_samples=8, seed=3)
    pm = MisfitProblem(precision="mixed", **kw)
    try:
        F = misfit_function()
        psi0 = pm.initial_psi().requires_grad_(True)
        J = F.apply(psi0, pm)
        J.backward()
        _, g = pm.value_and_gradient(psi0.detach())
        scale = float(g.abs().max())
        assert float((psi0.grad - g).abs().max()) <= 1e-12 * scale
    finally:
        pm.close()


def test_misfit_refuses_other_steppers_and_the_filter():
    from spectre_gb300.dgsw import DgswError
    with DgEvolution([Brick((2, 2, 2))], 4, time_stepper="adams_bashforth") as ev:
        ev.set_samples(np.array([[1.0, 1.0, 1.0]]))
        with pytest.raises(DgswError):
            ev.misfit_forward(np.zeros((1, 1)), 2, 1e-3)
    with DgEvolution([Brick((2, 2, 2))], 4) as ev:
        ev.set_samples(np.array([[1.0, 1.0, 1.0]]))
        ev.set_exponential_filter(36.0, 32)
        with pytest.raises(DgswError):
            ev.misfit_forward(np.zeros((1, 1)), 2, 1e-3)
