"""Misfit objective and its discrete adjoint behind torch.autograd.Function.

The control is the initial Psi field of one evolution (one periodic brick,
uniform LGL extent).  J(Psi0) = sum over windows m and sample points s of
(Psi(x_s, t_m) - target_ms)^2, with Psi sampled every `steps_per_window`
SSP-RK3 steps.  The gradient comes from the hand-written discrete adjoint of
the DG step (dgsw_misfit_adjoint); the step map is linear, so the reverse
sweep needs the recorded residuals only.  precision="mixed" runs the forward
and the adjoint sweep in mixed precision (FP64 states, FP32 increments); the
targets and the base state always come from an FP64 run.
"""
from __future__ import annotations

import math

import numpy as np

from .dgsw import Brick, DgEvolution, PRECISION_FP64, PRECISION_MIXED

TWO_PI = 2.0 * math.pi


def psi_view(state, n_elem: int, n: int):
    """Psi component of a state vector, shape [n_elem, n^3] (a view)."""
    return state.reshape(n_elem, 5, n ** 3)[:, 0, :]


class MisfitProblem:
    """Owns one DgEvolution (FP64 or mixed precision), the fixed (Pi, Phi) of
    the initial state, the sample points and the target trace."""

    def __init__(self, elements=(8, 8, 8), points=8, dt=5e-4, steps=2000, steps_per_window=10,
                 n_samples=64, seed=4, device=0, precision="fp64"):
        import torch
        prec = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED}[precision]
        self.precision = precision
        self.ev = DgEvolution([Brick(elements)], points, precision=PRECISION_FP64, device=device)
        self.n = points
        self.dt = dt
        self.steps_per_window = steps_per_window
        self.n_windows = steps // steps_per_window
        rng = np.random.default_rng(seed)
        # interior sample points, away from the outer faces of the cube
        self.xyz = rng.uniform(0.5, TWO_PI - 0.5, (n_samples, 3))
        self.ev.set_samples(self.xyz)
        # target trace: forward run from a seeded perturbation of the pulse
        amp = rng.uniform(0.5, 1.5)
        width = rng.uniform(0.3, 0.8)
        self.target_params = np.array([[amp, width, math.pi, math.pi, math.pi]])
        self.ev.set_initial_data("gaussian", self.target_params)
        samples = []
        for _ in range(self.n_windows):
            self.ev.step(self.steps_per_window, dt)
            samples.append(self.ev.sample_psi())
        self.targets = np.array(samples)
        # base state of the control run: unit Gaussian pulse, width 0.5
        self.base_params = np.array([[1.0, 0.5, math.pi, math.pi, math.pi]])
        self.ev.set_initial_data("gaussian", self.base_params)
        self.base_state = torch.tensor(self.ev.get_state(), dtype=torch.float64,
                                       device="cuda:%d" % device)
        self.n_elem = self.ev.n_elements
        if prec != PRECISION_FP64:
            self.ev.close()
            self.ev = DgEvolution([Brick(elements)], points, precision=prec, device=device)
            self.ev.set_samples(self.xyz)

    def initial_psi(self):
        return psi_view(self.base_state, self.n_elem, self.n).clone()

    def _state(self, psi0):
        u = self.base_state.clone()
        psi_view(u, self.n_elem, self.n).copy_(psi0.reshape(self.n_elem, -1))
        return u

    def value(self, psi0) -> float:
        self.ev.set_state(self._state(psi0))
        return self.ev.misfit_forward(self.targets, self.steps_per_window, self.dt)

    def value_and_gradient(self, psi0):
        J = self.value(psi0)
        g = self.ev.misfit_adjoint()
        return J, psi_view(g, self.n_elem, self.n).clone()

    def tangent_linear(self, psi0, direction) -> float:
        """dJ along `direction` by forward-mode differentiation: the linear
        step propagates the perturbation, dJ = sum 2 r_ms (S du)_ms."""
        # residuals of the control run
        self.ev.set_state(self._state(psi0))
        res = []
        for m in range(self.n_windows):
            self.ev.step(self.steps_per_window, self.dt)
            res.append(self.ev.sample_psi() - self.targets[m])
        du = self.base_state.clone().zero_()
        psi_view(du, self.n_elem, self.n).copy_(direction.reshape(self.n_elem, -1))
        self.ev.set_state(du)
        acc = 0.0
        for m in range(self.n_windows):
            self.ev.step(self.steps_per_window, self.dt)
            acc += 2.0 * float(np.dot(res[m], self.ev.sample_psi()))
        return acc

    def close(self):
        self.ev.close()


def misfit_function():
    """torch.autograd.Function computing J(psi0) with the adjoint gradient."""
    import torch

    class MisfitFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, psi0, problem):
            J, g = problem.value_and_gradient(psi0.detach())
            ctx.save_for_backward(g)
            return torch.tensor(J, dtype=torch.float64, device=psi0.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None

    return MisfitFunction
