"""Pins the oracle's CurvedScalarWave pieces to the reference's golden
functions and closed forms (configuration 5)."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CG = json.load(open(os.path.join(HERE, "golden", "curved_golden.json")))


def test_curved_upwind_penalty_golden(oracle):
    pk = []
    for side, ref in zip(CG["sides"], CG["packaged"]):
        s = {k: np.array(v) for k, v in side.items()}
        p, _ = oracle.csw_package(s["psi"], s["pi"], s["phi"], s["lapse"], s["shift"],
                                  s["gamma1"], s["gamma2"], s["normal"], s["normal_vector"])
        np.testing.assert_allclose(p, np.array(ref), rtol=1e-14, atol=1e-15)
        pk.append(p)
    bt = oracle.csw_boundary_terms(pk[0], pk[1])
    np.testing.assert_allclose(bt, np.array(CG["boundary_terms"]), rtol=1e-13, atol=1e-14)


def test_cpsr_golden(oracle):
    s = {k: np.array(v) for k, v in CG["sides"][0].items()}
    c = {k: np.array(v) for k, v in CG["cpsr"].items()}
    n = CG["npts"]
    # d_phi from the fixture is [i][j][p] = d_i Phi_j
    out = oracle.csw_cpsr(s["psi"], s["pi"], s["phi"], s["lapse"], s["shift"], s["gamma1"],
                          s["gamma2"], s["normal"], s["normal_vector"], c["xyz"], c["d_psi"],
                          c["d_pi"], c["d_phi"].reshape(9, n), c["dt_psi"], c["dt_pi"],
                          c["dt_phi"])
    np.testing.assert_allclose(out, c["out"], rtol=1e-13, atol=1e-14)


def test_kerr_schild_background_identities(oracle):
    # closed forms of Test_KerrSchild.cpp; here checked against independent
    # identities: inverse metric x metric = 1, lapse/shift from the 4-metric,
    # derivatives against central differences
    rng = np.random.default_rng(0)
    M = 1.0
    x = rng.uniform(2.5, 15.0, (3, 40)) * rng.choice([-1, 1], (3, 40))
    bg = oracle.ks_background(x, M)
    r = np.linalg.norm(x, axis=0)
    l = x / r
    H = M / r
    g = np.eye(3)[:, :, None] + 2 * H * l[:, None, :] * l[None, :, :]
    idx = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    gi = np.zeros((3, 3, 40))
    for q, (i, j) in enumerate(idx):
        gi[i, j] = gi[j, i] = bg[16 + q]
    prod = np.einsum("ijp,jkp->ikp", gi, g)
    np.testing.assert_allclose(prod, np.broadcast_to(np.eye(3)[:, :, None], prod.shape),
                               atol=1e-14)
    np.testing.assert_allclose(bg[0], 1 / np.sqrt(1 + 2 * H), rtol=1e-15)
    np.testing.assert_allclose(bg[1:4], 2 * H / (1 + 2 * H) * l, rtol=1e-14)
    h = 1e-6
    for i in range(3):
        dx = np.zeros((3, 1))
        dx[i] = h
        fd = (oracle.ks_background(x + dx, M) - oracle.ks_background(x - dx, M)) / (2 * h)
        np.testing.assert_allclose(bg[4 + i], fd[0], rtol=1e-7, atol=1e-10)  # d_i lapse
        for j in range(3):
            np.testing.assert_allclose(bg[7 + 3 * i + j], fd[1 + j], rtol=1e-7, atol=1e-10)


def test_curved_time_derivative_flat_limit(oracle):
    # M = 0 background (lapse 1, no shift, flat metric): the curved equations
    # reduce to the flat ScalarWave ones with gamma2 (TimeDerivative.cpp)
    rng = np.random.default_rng(2)
    n = 25
    bg = np.zeros((26, n))
    bg[0] = 1.0
    bg[16] = bg[19] = bg[21] = 1.0
    d_psi, d_pi = rng.normal(size=(3, n)), rng.normal(size=(3, n))
    d_phi = rng.normal(size=(9, n))
    pi, phi = rng.normal(size=n), rng.normal(size=(3, n))
    g2 = 0.7
    dt = oracle.csw_time_derivative(d_psi, d_pi, d_phi, pi, phi, bg, 0.0, g2)
    np.testing.assert_allclose(dt[0], -pi, rtol=1e-15)
    np.testing.assert_allclose(dt[1], -(d_phi[0] + d_phi[4] + d_phi[8]), rtol=1e-14)
    for i in range(3):
        np.testing.assert_allclose(dt[2 + i], -d_pi[i] + g2 * (d_psi[i] - phi[i]), rtol=1e-14)


# ---------------- spherical shell of six wedges ----------------

def _shell(oracle, **kw):
    args = dict(r_inner=1.9, r_outer=20.0, ref_ang=1, ref_rad=1, n=6, mass=1.0, gamma1=0.0,
                gamma2=1.0)
    args.update(kw)
    return oracle.shell(**args)


def test_shell_geometry(oracle):
    s = _shell(oracle, n=10)
    E = oracle.shell_num_elements(s)
    assert E == 6 * 4 * 2
    xyz, ij = oracle.shell_geometry(s)
    r = np.sqrt((xyz ** 2).sum(1))
    assert abs(r.min() - 1.9) < 1e-13 and abs(r.max() - 20.0) < 1e-12
    # the inverse Jacobian inverts the spectral derivative of the coordinates
    # (the map is smooth, so the LGL derivative is accurate to ~1e-8 at N=10)
    n = s.n
    D = oracle.diff_matrix(n)
    X = xyz.reshape(E, 3, n, n, n)  # [e][i][k][j][i_xi]
    jac = np.empty((E, 3, 3, n ** 3))  # dx^i / dxi^a
    jac[:, :, 0] = np.einsum("pq,ecjkq->ecjkp", D, X).reshape(E, 3, -1)
    jac[:, :, 1] = np.einsum("pq,eckql->eckpl", D, X).reshape(E, 3, -1)
    jac[:, :, 2] = np.einsum("pq,ecqjl->ecpjl", D, X).reshape(E, 3, -1)
    IJ = ij.reshape(E, 3, 3, -1)  # [e][a][i]
    prod = np.einsum("eaip,eibp->eabp", IJ, jac)
    err = np.abs(prod - np.eye(3)[None, :, :, None]).max()
    assert err < 1e-6, err


def test_shell_connectivity(oracle):
    s = _shell(oracle, ref_ang=1, ref_rad=2, n=5)
    E = oracle.shell_num_elements(s)
    nbr, perm, ids = oracle.shell_connectivity(s)
    assert (nbr == -1).sum() == 6 * 4 and (nbr == -2).sum() == 6 * 4
    assert (nbr[:, 4] == -1).sum() == 24 and (nbr[:, 5] == -2).sum() == 24
    assert len(set(ids.tolist())) == E
    xyz, _ = oracle.shell_geometry(s)
    n = s.n

    def face_idx(d, upper, a, b):
        sl = n - 1 if upper else 0
        return [sl + n * (a + n * b), a + n * (sl + n * b), a + n * (b + n * sl)][d]

    for e in range(E):
        for d in range(6):
            nb = nbr[e, d]
            if nb < 0:
                continue
            back = [fd for fd in range(6) if nbr[nb, fd] == e]
            assert len(back) == 1
            fd = back[0]
            p = perm[e, d]
            assert sorted(p.tolist()) == list(range(n * n))
            # the permutation composed with the neighbour's one is the identity
            assert (perm[nb, fd][p] == np.arange(n * n)).all()
            for q in range(n * n):
                mine = face_idx(d // 2, d % 2, q % n, q // n)
                theirs = face_idx(fd // 2, fd % 2, p[q] % n, p[q] // n)
                assert np.abs(xyz[e, :, mine] - xyz[nb, :, theirs]).max() < 1e-12


def _gaussian_shell_dt(oracle, xyz, gamma1, gamma2, r0=8.0, w=1.0):
    X = xyz.transpose(1, 0, 2).reshape(3, -1)
    r = np.sqrt((X ** 2).sum(0))
    psi = np.exp(-(r - r0) ** 2 / w ** 2)
    f = -2 * (r - r0) / w ** 2 * psi
    fr = (-2 / w ** 2 + 4 * (r - r0) ** 2 / w ** 4) * psi
    dpsi = f * X / r
    dphi = np.zeros((9, X.shape[1]))
    for i in range(3):
        for j in range(3):
            dphi[3 * i + j] = fr * X[i] * X[j] / r ** 2 + f * ((i == j) - X[i] * X[j] / r ** 2) / r
    bg = oracle.ks_background(X, 1.0)
    zero = np.zeros(X.shape[1])
    return oracle.csw_time_derivative(dpsi, np.zeros((3, X.shape[1])), dphi, zero, dpsi, bg,
                                      gamma1, gamma2)


def test_shell_rhs_converges_to_analytic(oracle):
    # for a smooth field sampled exactly the face corrections vanish (both
    # sides agree) and the DG time derivative converges spectrally to the
    # pointwise one evaluated with exact derivatives
    errs = []
    for n in (6, 8, 10, 12):
        s = _shell(oracle, ref_ang=1, ref_rad=3, n=n)
        xyz, _ = oracle.shell_geometry(s)
        u = oracle.shell_initial_data(s, 8.0, 1.0)
        du, ok = oracle.shell_rhs(s, u)
        assert ok
        exact = _gaussian_shell_dt(oracle, xyz, 0.0, 1.0)
        errs.append(np.abs(du.transpose(1, 0, 2).reshape(5, -1) - exact).max())
    assert all(a > 4.0 * b for a, b in zip(errs, errs[1:])), errs
    assert errs[-1] < 1e-3, errs


def test_shell_constant_state_and_boundaries(oracle):
    # constant Psi is a solution of the interior equations; only the outer
    # radiation condition (which demands Psi ~ 1/r falloff) corrects Pi there
    s = _shell(oracle, ref_ang=0, ref_rad=1, n=5)
    E = oracle.shell_num_elements(s)
    u = np.zeros((E, 5, s.n ** 3))
    u[:, 0] = 1.0
    du, ok = oracle.shell_rhs(s, u)
    assert ok
    xyz, _ = oracle.shell_geometry(s)
    r = np.sqrt((xyz ** 2).sum(1))
    outer = np.abs(r - 20.0) < 1e-9
    assert np.abs(du[:, [0, 2, 3, 4]]).max() < 1e-12
    assert np.abs(du[:, 1][~outer]).max() < 1e-12
    # CPSR: dt Pi correction = (2 Psi / r^2) / lapse + gamma2 * 0 - dt Pi
    lapse = 1.0 / np.sqrt(1.0 + 2.0 / 20.0)
    np.testing.assert_allclose(du[:, 1][outer], 2.0 / 400.0 / lapse, rtol=1e-12)
    # excision: an inner sphere outside the horizon has incoming speeds
    s_bad = _shell(oracle, r_inner=3.0, ref_ang=0, ref_rad=0, n=4)
    _, ok = oracle.shell_rhs(s_bad, np.zeros((6, 5, 64)))
    assert not ok


def test_shell_evolution_stable(oracle):
    s = _shell(oracle, ref_ang=0, ref_rad=1, n=6)
    u = oracle.shell_initial_data(s, 8.0, 1.0)
    u1, ok = oracle.shell_evolve(s, u, 1e-2, 20)
    assert ok and np.isfinite(u1).all()
    assert np.abs(u1).max() < 2.0 * np.abs(u).max()
    # linear: evolving a scaled state gives the scaled result
    u2, _ = oracle.shell_evolve(s, 3.0 * u, 1e-2, 20)
    np.testing.assert_allclose(u2, 3.0 * u1, rtol=1e-12, atol=1e-13)
