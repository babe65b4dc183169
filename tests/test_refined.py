"""h-nonconforming refined block lattices through the C ABI.

CPU: element ids, neighbour slots and mortar sizes bit-exact with the oracle;
half-interval projections within 1e-14 of the oracle's.  GPU: FP64
right-hand side on random states (2:1 faces in every direction, with and
without gamma2) and steps against the oracle (<= 1e-12 / 1e-11 relative per
variable); a smooth plane wave converges across the 2:1 faces."""
import math

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import DgEvolution, RefinedBrick

LATTICES = [((2, 2, 2), [1, 2, 1, 1, 2, 1, 1, 2]), ((2, 1, 1), [0, 1]),
            ((3, 1, 2), [1, 0, 1, 0, 1, 0])]


@pytest.mark.parametrize("case", range(len(LATTICES)))
def test_refined_maps_bit_exact(dgsw_lib, oracle, case):
    blocks, levels = LATTICES[case]
    rb = RefinedBrick(blocks, levels)
    r = oracle.refined(blocks, levels)
    ids, nbr, mort, fits = dgsw.index_maps(rb, 5)
    slots, sizes = dgsw.refined_mortars(rb, 5)
    oids, onbr, oms = r.index_maps()
    assert fits and ids.tolist() == oids.tolist()
    assert (slots == onbr).all() and (sizes == oms).all()
    assert (nbr == onbr[:, :, 0]).all()


def test_refined_unbalanced_rejected(dgsw_lib):
    with pytest.raises(dgsw.DgswError):
        dgsw.index_maps(RefinedBrick((2, 1, 1), [0, 2]), 4)


@pytest.mark.parametrize("n", [2, 5, 8, 12])
def test_half_projections_match_oracle(dgsw_lib, oracle, n):
    for up in (0, 1):
        P, R = dgsw.half_projections(n, up)
        oP, oR = oracle.proj_half(n, up)
        # different FMA contraction on different hosts: a few ulps of the
        # largest entry
        np.testing.assert_allclose(P, oP, rtol=0, atol=1e-14)
        np.testing.assert_allclose(R, oR, rtol=0, atol=1e-14)


def _rel(a, b, n):
    a = np.asarray(a).reshape(-1, 5, n ** 3)
    b = np.asarray(b).reshape(-1, 5, n ** 3)
    return max(np.abs(a[:, v] - b[:, v]).max() / np.abs(b[:, v]).max() for v in range(5))


@pytest.mark.gpu
@pytest.mark.parametrize("case,n", [(0, 4), (0, 7), (1, 10), (2, 6), (2, 12)])
def test_gpu_refined_rhs_matches_oracle(oracle, case, n):
    blocks, levels = LATTICES[case]
    r = oracle.refined(blocks, levels)
    u = np.random.default_rng(n).uniform(-1, 1, r.num_elements() * 5 * n ** 3)
    for g2 in (0.0, 0.7):
        with DgEvolution(RefinedBrick(blocks, levels), n, gamma2=g2) as ev:
            got = ev.rhs(u)
        assert _rel(got, r.rhs(n, u, gamma2=g2), n) <= 1e-12


@pytest.mark.gpu
def test_gpu_refined_steps_match_oracle(oracle):
    blocks, levels = LATTICES[0]
    n, dt = 6, 1e-3
    r = oracle.refined(blocks, levels)
    u = r.plane_wave(n, [1, 1, 1]).ravel()
    ref = r.evolve(n, u, dt, 10)
    with DgEvolution(RefinedBrick(blocks, levels), n) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        np.testing.assert_allclose(ev.get_state(), u, rtol=0, atol=1e-14)
        ev.step(10, dt)
        assert _rel(ev.get_state(), ref, n) <= 1e-11
        ev.set_state(u)
        for _ in range(10):
            for k in range(3):
                ev.substep(k, dt)
        assert _rel(ev.get_state(), ref, n) <= 1e-11


@pytest.mark.gpu
def test_gpu_refined_plane_wave_converges():
    errs = []
    for n in (4, 6, 8):
        with DgEvolution(RefinedBrick((2, 2, 2), [1, 2, 1, 1, 2, 1, 1, 2]), n) as ev:
            ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
            ev.step(50, 5e-4)
            errs.append(ev.observe_plane_wave_errors([1.0, 1.0, 1.0], 50 * 5e-4)
                        ["L2Norm(Error(Psi))"])
    assert errs[0] > 10 * errs[1] > 100 * errs[2], errs


@pytest.mark.gpu
def test_gpu_refined_gaussian_initial_data(oracle):
    # a refined lattice is one instance: one (A, width, centre) row sets the
    # Gaussian pulse on every element (evaluated at the oracle's coordinates)
    blocks, levels = LATTICES[0]
    n = 5
    r = oracle.refined(blocks, levels)
    xyz = r.coords(n)
    A, w, c = 1.3, 0.8, np.array([1.0, 2.0, 3.0])
    dx = xyz - c[None, :, None]
    psi = A * np.exp(-(dx ** 2).sum(axis=1) / (w * w))
    want = np.zeros((xyz.shape[0], 5, n ** 3))
    want[:, 0] = psi
    for d in range(3):
        want[:, 2 + d] = -2.0 * dx[:, d] / (w * w) * psi
    with DgEvolution(RefinedBrick(blocks, levels), n) as ev:
        ev.set_initial_data("gaussian", np.array([[A, w, *c]]))
        np.testing.assert_allclose(ev.get_state(), want.ravel(), rtol=0, atol=1e-13)
