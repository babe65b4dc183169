"""dgsw_set_guards: the Cfl rejection (DGSW_ERR_CFL) and the NaN / Inf
report (DGSW_ERR_NOT_FINITE) of dgsw_step; dgsw_check_finite."""
import math

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick, DgEvolution, DgswError

pytestmark = pytest.mark.gpu


def test_cfl_guard_refuses_long_steps_before_any_work():
    b = [Brick((6, 6, 6))]
    n = 6
    cfl = dgsw.cfl_steps(b, n, 1.0).min()
    with DgEvolution(b, n) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        u0 = ev.get_state()
        ev.set_guards(cfl_safety_factor=1.0)
        with pytest.raises(DgswError) as exc:
            ev.step(1, 1.01 * cfl)
        assert "Cfl" in str(exc.value)
        assert np.array_equal(ev.get_state(), u0)  # nothing ran
        ev.step(2, 0.99 * cfl)
        ev.set_guards(0.0)  # off again
        ev.step(1, 1.01 * cfl)


def test_cfl_guard_uses_each_element_step_level():
    b = [Brick((4, 4, 4))]
    n = 5
    cfl = dgsw.cfl_steps(b, n, 1.0, time_stepper="adams_bashforth", order=3)
    levels = np.zeros(64, np.int32)
    levels[::2] = 1
    with DgEvolution(b, n, time_stepper="adams_bashforth", order=3, step_levels=levels) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        ev.set_guards(cfl_safety_factor=1.0)
        # level-1 elements step slab / 2: a slab of 1.5 cfl is fine for
        # them and too long for the level-0 ones
        with pytest.raises(DgswError):
            ev.step(1, 1.5 * cfl.min())
        ev.step(1, 0.9 * cfl.min())


def test_finite_guard_reports_nan():
    b = [Brick((4, 4, 4))]
    n = 4
    with DgEvolution(b, n) as ev:
        ev.set_initial_data("plane_wave", [1.0, 1.0, 1.0])
        u = ev.get_state()
        assert ev.first_non_finite_element() == -1
        u[5 * 5 * n ** 3 + 17] = np.nan  # element 5, Psi
        ev.set_state(u)
        assert ev.first_non_finite_element() == 5
        ev.step(1, 1e-3)  # no guard: no report
        ev.set_state(u)
        ev.set_guards(check_finite=True)
        with pytest.raises(DgswError) as exc:
            ev.step(1, 1e-3)
        assert "NaN or Inf" in str(exc.value)
