"""Pins the CPU oracle to the reference's own golden vectors and known answers."""
import json
import math
import os

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick

HERE = os.path.dirname(os.path.abspath(__file__))
LGL = json.load(open(os.path.join(HERE, "golden", "lgl_golden.json")))
UPW = json.load(open(os.path.join(HERE, "golden", "upwind_golden.json")))


@pytest.mark.parametrize("n", sorted(int(k) for k in LGL["points_weights"]))
def test_lgl_points_weights_golden(oracle, n):
    # Test_LegendreGaussLobatto.cpp: points with Approx (1e-14), weights 1e-8
    g = LGL["points_weights"][str(n)]
    x, w = oracle.lgl(n)
    np.testing.assert_allclose(x, g["x"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(w, g["w"], rtol=1e-8, atol=1e-8)


@pytest.mark.parametrize("n", sorted(int(k) for k in LGL["diff_matrix"]))
def test_diff_matrix_golden(oracle, n):
    # Test_LegendreGaussLobatto.cpp DiffMatrix: Approx with margin 1e-13
    D = oracle.diff_matrix(n)
    G = np.array(LGL["diff_matrix"][str(n)])
    np.testing.assert_allclose(D, G, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("n", sorted(int(k) for k in LGL["modal_to_nodal"]))
def test_vandermonde_golden(oracle, n):
    np.testing.assert_allclose(oracle.vandermonde(n), np.array(LGL["modal_to_nodal"][str(n)]),
                               rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(oracle.inv_vandermonde(n),
                               np.array(LGL["nodal_to_modal"][str(n)]), rtol=1e-12, atol=1e-13)


def test_lgl_against_numpy_legendre(oracle):
    # Python/Test_Spectral.py: interior LGL nodes are the roots of P_{N-1}'
    from numpy.polynomial import legendre
    for n in range(3, 21):
        coefs = np.zeros(n)
        coefs[-1] = 1
        roots = np.sort(legendre.Legendre(coefs).deriv().roots())
        x, _ = oracle.lgl(n)
        np.testing.assert_allclose(x[1:-1], roots, atol=1e-13)


def test_diff_matrix_polynomial_exactness(oracle):
    # Test_PartialDerivatives.cpp: exact for polynomials of degree < N
    for n in range(2, 13):
        x, _ = oracle.lgl(n)
        D = oracle.diff_matrix(n)
        for p in range(n):
            np.testing.assert_allclose(D @ x**p, p * x**max(p - 1, 0) if p else 0 * x,
                                       atol=1e-11 * max(1, p * p))


def test_projection_exactness(oracle):
    # Test_Projection.cpp: face->mortar interpolation is exact for the face
    # polynomial; mortar->face restriction recovers it (modal truncation).
    rng = np.random.default_rng(1)
    for ne in range(2, 11):
        for nm in range(ne, 12):
            xe, _ = oracle.lgl(ne)
            xm, _ = oracle.lgl(nm)
            coef = rng.normal(size=ne)
            fe = np.polynomial.legendre.legval(xe, coef)
            fm = np.polynomial.legendre.legval(xm, coef)
            P = oracle.proj_face_to_mortar(ne, nm)
            np.testing.assert_allclose(P @ fe, fm, atol=1e-12)
            R = oracle.proj_mortar_to_face(ne, nm)
            np.testing.assert_allclose(R @ fm, fe, atol=1e-12)


def test_upwind_penalty_golden(oracle):
    # UpwindPenalty.py (pypp golden functions) on seeded inputs
    n = UPW["npts"]
    pk = []
    for inp, ref in zip(UPW["inputs"], UPW["packaged"]):
        p, ms = oracle.package(np.array(inp["psi"]), np.array(inp["pi"]),
                               np.array(inp["phi"]), np.array(inp["gamma2"]),
                               np.array(inp["normal"]))
        np.testing.assert_allclose(p, np.array(ref), rtol=1e-14, atol=1e-15)
        assert ms == 1.0
        pk.append(p)
    bt = oracle.boundary_terms(pk[0], pk[1])
    np.testing.assert_allclose(bt, np.array(UPW["boundary_terms"]), rtol=1e-14, atol=1e-15)
    sc = UPW["speeds_case"]
    bt2 = oracle.boundary_terms(np.array(sc["pkg_int"]), np.array(sc["pkg_ext"]))
    np.testing.assert_allclose(bt2, np.array(sc["boundary_terms"]), rtol=1e-14, atol=1e-15)
    assert bt.shape == (5, n)


def test_upwind_penalty_structure(oracle):
    # With char speeds (0, +1, -1) (no mesh velocity) the correction has
    # D_Psi = 0 and D_Phi = -n D_Pi for any gamma2 and unit normal: the
    # identity the fused kernels use (UpwindPenalty.cpp:145-202).
    rng = np.random.default_rng(3)
    n = 25
    nrm = rng.normal(size=(3, n))
    nrm /= np.linalg.norm(nrm, axis=0)
    a = [rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, (3, n)),
         rng.uniform(0, 2, n)]
    b = [rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, (3, n)),
         rng.uniform(0, 2, n)]
    pa, _ = oracle.package(*a, nrm)
    pb, _ = oracle.package(*b, -nrm)
    d = oracle.boundary_terms(pa, pb)
    np.testing.assert_allclose(d[0], 0.0, atol=0)
    np.testing.assert_allclose(d[2:], -nrm * d[1], atol=1e-14)
    wa = a[1] - np.einsum("in,in->n", nrm, a[2]) - a[3] * a[0]
    wb = b[1] - np.einsum("in,in->n", nrm, b[2]) - b[3] * b[0]
    np.testing.assert_allclose(d[1], 0.5 * (wa - wb), atol=1e-14)


def test_lift_known_answer(oracle):
    # Test_LiftFlux.cpp: lifted = -2/(L w_0) flux with w_0 = 2/(N(N-1)) on
    # an interval of length L; here via the full RHS of a field whose volume
    # derivative vanishes (constant fields) and whose neighbour differs.
    n = 4
    b = [Brick((2, 1, 1), (0, 0, 0), (2.0, 1.0, 1.0))]
    u = oracle.initial_data(b, n, "gaussian", oracle.gaussian_params(1)) * 0.0
    np_ = n ** 3
    # element 0: Pi = 1, element 1: Pi = 0 (piecewise constant)
    u[np_:2 * np_] = 1.0
    du = oracle.rhs(b, n, u)
    L = 1.0  # element width along x
    w0 = 2.0 / (n * (n - 1))
    # upper-x face of element 0: s=+1, w_int = 1, w_ext = 0: D_Pi = 1/2
    # lifted dt Pi = -N(N-1)/2 * (2/L) * 1/2 = -(1/(L w0)) * 1... both faces
    expected = -2.0 / (L * w0) * 0.5
    dpi = du[np_:2 * np_].reshape(n, n, n)
    np.testing.assert_allclose(dpi[:, :, n - 1], expected, rtol=1e-13)
    np.testing.assert_allclose(dpi[:, :, 0], expected, rtol=1e-13)
    np.testing.assert_allclose(dpi[:, :, 1:n - 1], 0.0, atol=1e-13)


def test_rk3_order_and_ssp(oracle):
    # Test_Rk3HesthavenSsp.cpp: third order; SSP (Delta t = 1 stays bounded)
    lam = -1.0

    def integrate(dt, steps):
        y = np.array([1.0])
        for _ in range(steps):
            u0 = y.copy()
            u1 = oracle.rk3_substep(0, dt, u0, u0, lam * u0)
            u2 = oracle.rk3_substep(1, dt, u0, u1, lam * u1)
            y = oracle.rk3_substep(2, dt, u0, u2, lam * u2)
        return y[0]

    errs = [abs(integrate(1.0 / k, k) - math.exp(-1.0)) for k in (20, 40, 80)]
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(2.9 < r < 3.1 for r in rates), rates
    # y' = -y with dt = 1: |amplification| <= 1 (strong stability)
    assert abs(integrate(1.0, 1)) <= 1.0


def test_index_maps_known(oracle):
    # 4x4x4 single block (refinement 2): x outer, z inner; periodic wrap
    ids, nbr, ijk, inst, fits = oracle.index_maps([Brick((4, 4, 4))])
    assert fits and len(ids) == 64
    assert tuple(ijk[1]) == (0, 0, 1) and tuple(ijk[4]) == (0, 1, 0)
    assert tuple(ijk[16]) == (1, 0, 0)
    # element 0's lower-xi neighbour is the periodic image at ix = 3
    assert nbr[0, 0] == 48 and nbr[0, 1] == 16 and nbr[0, 4] == 3
    # ElementId bits: index_xi << 16 | ref_xi << 28 | ... for element (1,2,3)
    e = 16 * 1 + 4 * 2 + 3
    expect = (1 << 16) | (2 << 28) | (2 << 32) | (2 << 44) | (3 << 48) | (2 << 60)
    assert int(ids[e]) == expect
    # 3x6x1: blocks (3,3,1) x-fastest, refinement (0,1,0)
    ids, nbr, ijk, inst, fits = oracle.index_maps([Brick((3, 6, 1))])
    assert len(ids) == 18
    assert tuple(ijk[0]) == (0, 0, 0) and tuple(ijk[1]) == (0, 1, 0)  # same block
    assert tuple(ijk[2]) == (1, 0, 0)                                 # next block (x)
    assert int(ids[2]) & 0xff == 1
    assert int(ids[1]) == (1 << 32) | (1 << 44)


def test_plane_wave_convergence(oracle):
    # A scaled-down plane-wave case (plane wave on [0, 2pi]^3, k=(1,1,1)): the DG
    # solution converges to the analytic wave at the spectral rate.
    errs = []
    for n in (4, 5, 6):
        b = [Brick((2, 2, 2))]
        u = oracle.initial_data(b, n, "plane_wave", [1.0, 1.0, 1.0])
        dt, steps = 2e-3, 25
        u = oracle.evolve(b, n, u, dt, steps)
        ua = oracle.initial_data(b, n, "plane_wave", [1.0, 1.0, 1.0], t=dt * steps)
        errs.append(np.max(np.abs(u - ua)))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-3
