"""Host logic of the Adams-Bashforth / local-time-stepping path (no GPU).

The product's coefficient functions are checked against the reference's
known answers, and the product's device schedule (the per-level coefficient
tables every launch applies) is executed here in numpy, launch by launch, the
way the kernel applies it: its result must equal the oracle's literal
per-element, per-mortar evolution."""
import json
import math
import os

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "adams_golden.json")))


@pytest.mark.parametrize("case", GOLDEN["lts"],
                         ids=lambda c: f'{c["case"]}:{c["step_start"]}-{c["step_end"]}')
def test_product_lts_coefficients_known_answers(case):
    # Test_AdamsLts.cpp:416-790, explicit cases (slab [-16, 16], unit ticks)
    local = [tuple(s) for s in case["local"]]
    remote = [tuple(s) for s in case["remote"]]
    got = dgsw.lts_coefficients(local, remote, case["step_start"], case["step_end"],
                                case["orders"], slab=32.0, ticks_per_slab=32)
    want = {(tuple(e["local"]), tuple(e["remote"])): e["coef"] for e in case["expected"]}
    assert set(got) == set(want)
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-13, abs=1e-14)


@pytest.mark.parametrize("order", range(1, 9))
def test_product_adams_coefficients(oracle, order):
    rng = np.random.default_rng(order)
    for _ in range(20):
        # random increasing control times, a step past the last one
        ticks = np.cumsum(rng.integers(1, 5, size=order)) - 40
        start = int(ticks[-1]) + int(rng.integers(0, 3))
        end = start + int(rng.integers(1, 6))
        got = dgsw.adams_coefficients(ticks, start, end, slab=0.3, ticks_per_slab=16)
        want = oracle.adams_coefficients(ticks, start, end, slab=0.3, ticks_per_slab=16)
        np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-13 * np.abs(want).max())


@pytest.mark.parametrize("ticks,start,end", [
    ([1, 2, 3, 4, 5, 6, 7, 0], 0, 8),      # order-8 self-start, first real step
    ([2, 3, 4, 5, 6, 7, 0, 8], 8, 16),     # ... and the second
    ([1, 2, 3, 0], 0, 4),
    ([-8, -4, 0, 2], 2, 4),                # 2:1 small steps
    ([0, 3, 5, 6, 9, 10, 12], 12, 17),     # ragged steps
])
def test_product_weights_exact(oracle, ticks, start, end):
    # the product's weights against exact rational integrals of the Lagrange
    # basis; the oracle (the reference's monomial expansion) is looser on the
    # non-monotonic self-start histories
    sp = pytest.importorskip("sympy")
    S, slab = 16, 0.01
    t = sp.symbols("t")
    pts = [sp.Rational(k, S) * sp.Rational(1, 100) for k in ticks]
    a, b = sp.Rational(start, S) / 100, sp.Rational(end, S) / 100
    exact = []
    for j in range(len(pts)):
        ell = sp.Integer(1)
        for m in range(len(pts)):
            if m != j:
                ell *= (t - pts[m]) / (pts[j] - pts[m])
        exact.append(float(sp.integrate(sp.expand(ell), (t, a, b))))
    exact = np.array(exact)
    got = dgsw.adams_coefficients(ticks, start, end, slab=slab, ticks_per_slab=S)
    assert np.abs(got - exact).max() <= 1e-14 * np.abs(exact).max()
    ref = oracle.adams_coefficients(ticks, start, end, slab=slab, ticks_per_slab=S)
    assert np.abs(ref - exact).max() <= 1e-11 * np.abs(exact).max()


def _face_points(n, d, upper):
    """volume indices of the face points (face index a + n b, transverse
    dimensions ascending)"""
    sl = n - 1 if upper else 0
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    a, b = a.ravel(), b.ravel()
    if d == 0:
        return sl + n * (a + n * b)
    if d == 1:
        return a + n * (sl + n * b)
    return a + n * (b + n * sl)


def run_schedule(oracle, bricks, n, u0, levels, order, slab, n_slabs, gamma2=0.0):
    """Applies the product's schedule the way the device kernel does."""
    ids, nbr, ijk, inst, _ = oracle.index_maps(bricks)
    E, npt = len(ids), n ** 3
    lv = np.asarray(levels, dtype=np.int64)
    counts = [int((lv == l).sum()) for l in range(4)]
    adj = np.zeros((4, 4), np.int32)
    for e in range(E):
        for f in range(6):
            adj[lv[e], lv[nbr[e, f]]] = 1
    jobs, S, ring = dgsw.adams_schedule(order, counts, adj, slab, n_slabs)
    jac = np.zeros((E, 3))
    for e in range(E):
        b = bricks[inst[e]]
        for d in range(3):
            jac[e, d] = 2.0 / ((b.upper[d] - b.lower[d]) / b.elements[d])
    faces = [[_face_points(n, d, up) for up in (0, 1)] for d in range(3)]
    u = np.array(u0, dtype=np.float64).reshape(E, 5, npt).copy()
    u_init = u.copy()
    F = np.zeros((ring, E, 5, npt))
    B = np.zeros((ring, E, 6, 2, n * n))  # P = Pi - gamma2 Psi, Q = Phi_d
    members = [np.where(lv == l)[0] for l in range(4)]
    by_launch = {}
    for j in jobs:
        by_launch.setdefault(j.launch, []).append(j)
    for key in sorted(by_launch):
        launch = by_launch[key]
        new = u.copy()
        for j in launch:
            if not j.update:
                continue
            for e in members[j.level]:
                for i in range(j.n_vol):
                    new[e] += j.vol_c[i] * F[j.vol_slot[i], e]
                for d in range(3):
                    for up in (0, 1):
                        s = 1.0 if up else -1.0
                        dr = 2 * d + up
                        nb = nbr[e, dr]
                        m = lv[nb]
                        own = sum(j.loc_c[m][i] * (B[j.loc_slot[m][i], e, dr, 0]
                                                   - s * B[j.loc_slot[m][i], e, dr, 1])
                                  for i in range(j.n_loc[m]))
                        ext = sum(j.rem_c[m][i] * (B[j.rem_slot[m][i], nb, dr ^ 1, 0]
                                                   - s * B[j.rem_slot[m][i], nb, dr ^ 1, 1])
                                  for i in range(j.n_rem[m]))
                        g = -0.25 * n * (n - 1) * jac[e, d]
                        p = faces[d][up]
                        new[e, 1, p] += g * (own - ext)
                        new[e, 2 + d, p] += -s * g * (own - ext)
        u = new
        for j in launch:
            if j.reset:
                u[members[j.level]] = u_init[members[j.level]]
        dudt = oracle.rhs(bricks, n, u.ravel(), gamma2=gamma2, volume_only=True).reshape(E, 5, npt)
        for j in launch:
            for e in members[j.level]:
                F[j.rec_slot, e] = dudt[e]
                for d in range(3):
                    for up in (0, 1):
                        p = faces[d][up]
                        B[j.rec_slot, e, 2 * d + up, 0] = u[e, 1, p] - gamma2 * u[e, 0, p]
                        B[j.rec_slot, e, 2 * d + up, 1] = u[e, 2 + d, p]
    return u.ravel(), len(by_launch), ring


CASES = [
    ("gts", [0] * 8, 1), ("gts", [0] * 8, 3), ("gts", [0] * 8, 4),
    ("2:1", [0, 1, 0, 1, 1, 0, 1, 0], 2), ("2:1", [0, 1, 0, 1, 1, 0, 1, 0], 3),
    ("4:1", [2, 1, 1, 0, 1, 0, 0, 0], 3), ("8:1", [3, 2, 1, 0, 2, 1, 0, 0], 2),
]


@pytest.mark.parametrize("name,levels,order", CASES, ids=[f"{c[0]}-k{c[2]}-{i}" for i, c in
                                                          enumerate(CASES)])
def test_schedule_reproduces_oracle(oracle, name, levels, order):
    n, gamma2 = 4, 0.7
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1.0, 1.0, 1.0])
    slab, n_slabs = 0.1, 3
    got, launches, ring = run_schedule(oracle, bricks, n, u0, levels, order, slab, n_slabs,
                                       gamma2=gamma2)
    want = oracle.evolve_adams(bricks, n, u0, slab, n_slabs, order, levels=levels,
                               gamma2=gamma2)
    assert np.linalg.norm(got - want) <= 1e-13 * np.linalg.norm(want)
    L = max(levels)
    # one launch per tick position: the start-up, then 2^L per slab
    startup = order * (order - 1) // 2 + (order - 1) + 1
    assert launches == startup + n_slabs * 2 ** L
    assert ring <= 2 * order + 2 ** L
