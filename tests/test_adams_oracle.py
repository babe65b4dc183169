"""The Adams-Bashforth / local-time-stepping oracle against the reference's
known answers (tests/golden/adams_golden.json, read from
Test_AdamsCoefficients.cpp and Test_AdamsLts.cpp) and against the orders of
accuracy the method promises."""
import json
import math
import os

import numpy as np
import pytest

from spectre_gb300.dgsw import Brick

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "adams_golden.json")))


@pytest.mark.parametrize("case", GOLDEN["variable"], ids=lambda c: str(c["control_times"]))
def test_variable_coefficients_known_answers(oracle, case):
    # Test_AdamsCoefficients.cpp:118-141 (exact rational answers)
    got = oracle.variable_coefficients(case["control_times"], case["step_start"],
                                       case["step_end"])
    np.testing.assert_allclose(got, case["expected"], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("order", range(1, 9))
def test_constant_step_dispatch(oracle, order):
    # Test_AdamsCoefficients.cpp:16-96: the constant-step table, the variable
    # formula on the same times, offsets and step scaling agree
    ticks = list(range(-order + 1, 1))
    const = oracle.adams_coefficients(ticks, 0, 1)
    var = oracle.variable_coefficients([float(t) for t in ticks], 0.0, 1.0)
    np.testing.assert_allclose(var, const, rtol=1e-11, atol=1e-13)
    assert abs(const.sum() - 1.0) < 1e-13
    scaled = oracle.adams_coefficients(ticks, 0, 1, slab=2.1, ticks_per_slab=1)
    np.testing.assert_array_equal(scaled, 2.1 * const)
    shifted = oracle.adams_coefficients([t + 7 for t in ticks], 7, 8)
    np.testing.assert_array_equal(shifted, const)


def _ids(steps):
    return [tuple(s) for s in steps]


@pytest.mark.parametrize("case", GOLDEN["lts"],
                         ids=lambda c: f'{c["case"]}:{c["step_start"]}-{c["step_end"]}')
def test_lts_coefficients_known_answers(oracle, case):
    # Test_AdamsLts.cpp:416-790, explicit cases.  The reference's slab is
    # [-16, 16] with integer times, so a tick is one time unit.
    local, remote = _ids(case["local"]), _ids(case["remote"])
    got = oracle.lts_coefficients(local, remote, case["step_start"], case["step_end"],
                                  case["orders"], slab=32.0, ticks_per_slab=32)
    want = {(tuple(e["local"]), tuple(e["remote"])): e["coef"] for e in case["expected"]}
    assert set(got) == set(want)
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-13, abs=1e-14)
    # the same step seen from the other side (Test_AdamsLts.cpp:398-406)
    lo, ro, so = case["orders"]
    flipped = oracle.lts_coefficients(remote, local, case["step_start"], case["step_end"],
                                      (ro, lo, so), slab=32.0, ticks_per_slab=32)
    assert {(b, a): v for (a, b), v in flipped.items()} == pytest.approx(got, rel=1e-13)


def _plane_wave_case(oracle, n=4):
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1.0, 1.0, 1.0])
    return bricks, u0


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_global_stepping_order(oracle, order):
    # self-start + AB(k) converges at order k against a time-resolved solution
    # of the same semi-discrete system
    n, T = 4, 0.4
    bricks, u0 = _plane_wave_case(oracle, n)
    ref = oracle.evolve(bricks, n, u0, T / 800, 800)
    errs = [np.abs(oracle.evolve_adams(bricks, n, u0, T / s, s, order) - ref).max()
            for s in (8, 16)]
    assert math.log2(errs[0] / errs[1]) > order - 0.5


@pytest.mark.parametrize("levels", [[0, 1, 0, 1, 1, 0, 1, 0], [2, 1, 1, 0, 1, 0, 0, 0]])
@pytest.mark.parametrize("order", [2, 3])
def test_local_stepping_order(oracle, levels, order):
    # 2:1 and 4:1 step ratios across faces keep the order of the method
    n, T = 4, 0.4
    bricks, u0 = _plane_wave_case(oracle, n)
    ref = oracle.evolve(bricks, n, u0, T / 800, 800)
    errs = [np.abs(oracle.evolve_adams(bricks, n, u0, T / s, s, order, levels=levels)
                   - ref).max() for s in (8, 16)]
    assert math.log2(errs[0] / errs[1]) > order - 0.5


def test_uniform_levels_are_global_stepping(oracle):
    # every element on the same level: the LTS boundary coefficients reduce
    # to the GTS ones (lts_coefficients_for_gts) and the run is GTS
    n = 4
    bricks, u0 = _plane_wave_case(oracle, n)
    a = oracle.evolve_adams(bricks, n, u0, 0.05, 3, 3)
    b = oracle.evolve_adams(bricks, n, u0, 0.05, 3, 3, levels=[0] * 8)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("order,lts", [(2, False), (3, False), (3, True)])
def test_curved_shell_order(oracle, order, lts):
    # the shell (curved UpwindPenalty across wedges, radiation condition in
    # dt u): AB(k), with or without 2:1 local stepping, converges at order k
    # against a time-resolved SSP-RK3 run of the same semi-discrete system
    s = oracle.shell(1.9, 20.0, 0, 1, 5, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5)
    T = 0.4
    ref, ok = oracle.shell_evolve(s, u0, T / 400, 400)
    levels = np.array([i % 2 for i in range(E)], np.int32) if lts else None
    errs = [np.abs(oracle.shell_evolve_adams(s, u0, T / k, k, order, levels=levels).ravel()
                   - ref.ravel()).max() for k in (8, 16)]
    assert math.log2(errs[0] / errs[1]) > order - 0.5


def test_extents_path_of_one_extent_is_the_uniform_path(oracle):
    # the oracle's per-element-extent system with every extent equal runs the
    # same arithmetic as the uniform one
    n = 4
    bricks, u0 = _plane_wave_case(oracle, n)
    levels = [0, 1, 0, 1, 1, 0, 1, 0]
    a = oracle.evolve_adams(bricks, n, u0, 0.05, 3, 3, levels=levels)
    b = oracle.evolve_adams_extents(bricks, [n] * 8, u0, 0.05, 3, 3, levels=levels)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("levels", [None, [0, 1, 0, 1, 1, 0, 1, 0], [2, 1, 1, 0, 1, 0, 0, 0]])
@pytest.mark.parametrize("order", [2, 3])
def test_extents_local_stepping_order(oracle, levels, order):
    # p-nonconforming faces (mortars at the larger extent) with 1:1, 2:1 and
    # 4:1 step ratios keep the order of the method against a time-resolved
    # SSP-RK3 run of the same semi-discrete system
    elem_n = [4, 5, 6, 4, 5, 4, 6, 5]
    T = 0.4
    bricks = [Brick((2, 2, 2), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    u0 = oracle.initial_data(bricks, elem_n, "plane_wave", [1.0, 1.0, 1.0])
    ref = oracle.evolve(bricks, elem_n, u0, T / 800, 800)
    errs = [np.abs(oracle.evolve_adams_extents(bricks, elem_n, u0, T / s, s, order,
                                               levels=levels) - ref).max() for s in (8, 16)]
    assert math.log2(errs[0] / errs[1]) > order - 0.5


def test_filtered_shell_alpha_zero_is_unfiltered(oracle):
    # alpha = 0 keeps every Legendre mode (F = I to rounding): the filtered
    # run of the curved executable's step actions equals the plain one
    s = oracle.shell(1.9, 20.0, 0, 1, 5, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5)
    levels = np.array([i % 2 for i in range(E)], np.int32)
    a = oracle.shell_evolve_adams(s, u0, 0.02, 3, 3, levels=levels)
    b = oracle.shell_evolve_adams(s, u0, 0.02, 3, 3, levels=levels, filter=(0.0, 8))
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_filtered_shell_damps_the_top_modes(oracle):
    # the filter after every step removes the top Legendre mode of every
    # element's state (exp(-36) ~ 2e-16), which the unfiltered run keeps
    n = 5
    s = oracle.shell(1.9, 20.0, 0, 1, n, 1.0, 0.0, 1.0)
    E = oracle.shell_num_elements(s)
    u0 = oracle.shell_initial_data(s, 8.0, 1.5)
    a = oracle.shell_evolve_adams(s, u0, 0.02, 3, 3)
    b = oracle.shell_evolve_adams(s, u0, 0.02, 3, 3, filter=(36.0, 8))
    Vi = oracle.inv_vandermonde(n)

    def top(u):
        modal = np.einsum("ai,bj,ck,evkji->evcba", Vi, Vi, Vi, u.reshape(E, 5, n, n, n))
        return max(np.abs(modal[..., n - 1]).max(), np.abs(modal[..., n - 1, :]).max(),
                   np.abs(modal[..., n - 1, :, :]).max())

    assert top(b) <= 1e-12 * np.abs(b).max()
    assert top(a) >= 1e-6 * np.abs(a).max()
