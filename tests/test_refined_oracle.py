"""h-nonconforming refined bricks in the oracle (2:1 block lattices).

Pins: the half-interval projections against the reference's own property
checks (Test_Projection.cpp: the restriction error is L2-orthogonal to every
polynomial the parent can hold, over both halves; prolongation is exact for
polynomials), their consistency sum_c R_c P_c = 1, the mortar maps (2:1
faces carry four half-size mortars on the coarse side and one full mortar on
the fine side, symmetric), bit-identity with the conforming oracle when every
block has the same level, spectral convergence of the nonconforming
right-hand side, and energy stability of the upwind scheme across 2:1 faces.
"""
import math

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick


@pytest.mark.parametrize("n", [2, 3, 5, 8, 12])
def test_half_projections_properties(oracle, n):
    x, _ = oracle.lgl(n)
    P0, R0 = oracle.proj_half(n, 0)
    P1, R1 = oracle.proj_half(n, 1)
    np.testing.assert_allclose(R0 @ P0 + R1 @ P1, np.eye(n), atol=5e-14)
    gx, gw = oracle.lg(min(2 * n + 2, 20))
    for upper, P, R in ((0, P0, R0), (1, P1, R1)):
        s = 1.0 if upper else -1.0
        for p in range(n):
            # prolongation: exact for polynomials of degree < n
            np.testing.assert_allclose(P @ x ** p, (0.5 * (x + s)) ** p, atol=1e-13)
            # restriction of the child polynomial g(xi) = xi^p living on one half
            c = R @ x ** p
            V = np.array([[np.prod([(t - x[m]) / (x[j] - x[m]) for m in range(n) if m != j])
                           for j in range(n)] for t in gx])  # Lagrange basis at gx
            parent_at = lambda t: V_at(t) @ c  # noqa: E731

            def V_at(t):
                return np.array([[np.prod([(tt - x[m]) / (x[j] - x[m]) for m in range(n)
                                           if m != j]) for j in range(n)] for tt in t])
            for k in range(n):
                # int_{-1}^{1} (parent - g chi_half) x^k dx = 0
                self_x = 0.5 * (gx + s)  # quadrature points of the half
                err_self = parent_at(self_x) - gx ** p
                other_x = 0.5 * (gx - s)
                err_other = parent_at(other_x)
                integ = 0.5 * (gw @ (err_self * self_x ** k) + gw @ (err_other * other_x ** k))
                assert abs(integ) < 1e-12, (n, upper, p, k, integ)
            del V




def test_refined_index_maps_2to1(oracle):
    r = oracle.refined((2, 2, 2), [1, 2, 1, 1, 2, 1, 1, 2])
    ids, nbr, ms = r.index_maps()
    E = r.num_elements()
    assert E == 5 * 8 + 3 * 64 and len(set(ids.tolist())) == E
    fine_to_coarse = coarse_to_fine = 0
    for e in range(E):
        for d in range(6):
            slots = [k for k in range(4) if nbr[e, d, k] >= 0]
            assert len(slots) in (1, 4)
            for k in slots:
                nb = nbr[e, d, k]
                back = [(d2, k2) for d2 in range(6) for k2 in range(4) if nbr[nb, d2, k2] == e]
                assert len(back) == 1 and back[0][0] == d ^ 1
                if len(slots) == 4:
                    coarse_to_fine += 1
                    assert (ms[e, d, k] > 0).all()
                    assert len([s for s in range(4) if nbr[nb, d ^ 1, s] >= 0]) == 1
                else:
                    assert (ms[e, d, k] == 0).all()
                    if len([s for s in range(4) if nbr[nb, d ^ 1, s] >= 0]) == 4:
                        fine_to_coarse += 1
    assert coarse_to_fine == fine_to_coarse > 0
    bad = oracle.refined((2, 1, 1), [0, 2])
    with pytest.raises(RuntimeError):
        bad.index_maps()


def test_refined_conforming_equals_brick(oracle):
    # blocks of one level lay out exactly as the brick's b * 2^L lattice
    r = oracle.refined((3, 1, 1), [1] * 3)
    n = 5
    u = np.random.default_rng(0).uniform(-1, 1, r.num_elements() * 5 * n ** 3)
    a = r.rhs(n, u).ravel()
    b = oracle.rhs([Brick((6, 2, 2))], n, u)
    assert np.array_equal(a, b)


def test_refined_rhs_converges(oracle):
    r = oracle.refined((2, 2, 2), [1, 2, 1, 1, 2, 1, 1, 2])
    errs = []
    for n in (4, 6, 8, 10):
        u = r.plane_wave(n, [1, 1, 1])
        du = r.rhs(n, u)
        ph = r.coords(n).sum(1)
        om = math.sqrt(3.0)
        ex = np.zeros_like(u)
        ex[:, 0] = -om * np.cos(ph)
        ex[:, 1] = 3.0 * np.sin(ph)
        ex[:, 2:] = (om * np.sin(ph))[:, None]
        errs.append(np.abs(du - ex).max())
    assert all(a > 20 * b for a, b in zip(errs, errs[1:])), errs


def test_refined_upwind_energy_stable(oracle):
    r = oracle.refined((2, 1, 1), [0, 1])
    n = 6
    rng = np.random.default_rng(1)
    u = rng.uniform(-1, 1, (r.num_elements(), 5, n ** 3))
    _, w = oracle.lgl(n)
    W = np.einsum("i,j,k->kji", w, w, w).ravel()
    ids, _, _ = r.index_maps()
    xyz = r.coords(n)
    vol = np.array([np.prod([xyz[e, c].max() - xyz[e, c].min() for c in range(3)]) / 8.0
                    for e in range(r.num_elements())])

    def energy(v):
        return 0.5 * float(np.sum(vol[:, None] * W[None, :] * (v[:, 1:] ** 2).sum(1)))

    e0 = energy(u)
    for _ in range(5):
        u = r.evolve(n, u, 1e-3, 1)
        e1 = energy(u)
        assert e1 <= e0 * (1 + 1e-12)
        e0 = e1
