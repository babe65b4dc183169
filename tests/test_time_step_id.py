"""Time bookkeeping through the C ABI: TimeStepId and next_time_id.

dgsw_time_step_id / dgsw_next_time_id / dgsw_substep_time_fraction against
the oracle's exact-fraction restatement of TimeStepId (TimeStepId.cpp:19-98)
and Rk3HesthavenSsp::next_time_id (Rk3HesthavenSsp.cpp:36-48): every field
bit for bit, over many steps, across slab boundaries, with several steps per
slab and with time running backwards.  CPU only.
"""
from fractions import Fraction

import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import DgswError, Rk3HesthavenSsp


def _walk(oracle, start_id, sizes, stepper="rk3_hesthaven_ssp"):
    """Advances the product's and the oracle's ids together through the
    substeps of len(sizes) steps (sizes as (num, den) slab fractions)."""
    prod = dgsw.time_step_id(*start_id)
    slab_number, s0, s1, num, den, forward = start_id
    orc = oracle.TimeStepIdOracle(forward, slab_number, s0, s1, Fraction(num, den))
    assert prod.key() == orc.key()
    n_sub = 3 if stepper == "rk3_hesthaven_ssp" else 1
    seen = 0
    for num, den in sizes:
        for _ in range(n_sub):
            prod = dgsw.next_time_id(stepper, prod, num, den)
            if stepper == "rk3_hesthaven_ssp":
                orc = oracle.rk3_next_time_id(orc, Fraction(num, den))
            else:
                orc = orc.next_step(Fraction(num, den))
            assert prod.key() == orc.key(), (prod.key(), orc.key())
            seen += 1
    return prod, seen


def test_substep_fractions():
    assert Rk3HesthavenSsp().substep_time_fractions() == (0.0, 1.0, 0.5)


def test_rk3_one_step_per_slab(oracle):
    # slab = step = 1e-3 (the global stepping of the configurations): 200 steps
    end, seen = _walk(oracle, (0, 0.0, 1e-3, 0, 1, True), [(1, 1)] * 200)
    assert seen == 600
    assert end.slab_number == 200 and end.substep == 0
    # the substep times of one step: t, t + dt, t + dt/2
    first = dgsw.time_step_id(0, 0.0, 1e-3, 0, 1)
    a = Rk3HesthavenSsp().next_time_id(first, 1, 1)
    b = Rk3HesthavenSsp().next_time_id(a, 1, 1)
    assert (first.substep_time, a.substep_time, b.substep_time) == (0.0, 1e-3, 0.5 * 1e-3)


def test_rk3_several_steps_per_slab(oracle):
    # steps of 1/3, 1/6, 1/2 of the slab [0.3, 0.7], repeated across slabs
    _walk(oracle, (4, 0.3, 0.7, 0, 1, True), [(1, 3), (1, 6), (1, 2)] * 20)
    # starting part-way into a slab
    _walk(oracle, (0, -1.0, 2.5, 2, 5, True),
          [(1, 5), (2, 5)] + [(2, 5), (1, 5), (2, 5)] * 10 + [(1, 10)] * 30)


def test_rk3_time_runs_backwards(oracle):
    _walk(oracle, (0, 1.0, 2.0, 1, 1, False), [(-1, 4)] * 40)


def test_adams_bashforth_next_step(oracle):
    _walk(oracle, (0, 0.0, 0.25, 0, 1, True), [(1, 8)] * 64, stepper="adams_bashforth")


def test_start_at_slab_end_moves_to_next_slab(oracle):
    p = dgsw.time_step_id(7, 0.5, 1.5, 1, 1)
    o = oracle.TimeStepIdOracle(True, 7, 0.5, 1.5, Fraction(1))
    assert p.key() == o.key()
    assert (p.slab_number, p.slab_start, p.slab_end, p.step_num) == (8, 1.5, 2.5, 0)


def test_errors_where_the_reference_errors():
    first = dgsw.time_step_id(0, 0.0, 1.0, 1, 2)
    with pytest.raises(DgswError):  # the step leaves its slab
        dgsw.next_time_id("rk3_hesthaven_ssp", first, 2, 3)
    with pytest.raises(DgswError):  # against the direction of time
        dgsw.next_time_id("rk3_hesthaven_ssp", first, -1, 4)
    mid = dgsw.next_time_id("rk3_hesthaven_ssp", first, 1, 4)
    with pytest.raises(DgswError):  # the step size changes within a step
        dgsw.next_time_id("rk3_hesthaven_ssp", mid, 1, 8)
    with pytest.raises(DgswError):  # AdamsBashforth has one substep
        dgsw.next_time_id("adams_bashforth", mid, 1, 4)
    with pytest.raises(DgswError):  # a time outside its slab
        dgsw.time_step_id(0, 0.0, 1.0, 3, 2)
    with pytest.raises(DgswError):  # substep 3 of Rk3HesthavenSsp
        f = dgsw.ctypes.c_double()
        dgsw._check(dgsw.lib().dgsw_substep_time_fraction(0, 3, dgsw.ctypes.byref(f)))
