"""CurvedScalarWave on the Kerr-Schild shell: CUDA path vs the CPU FP64 oracle,
through the C ABI.

Tolerances: the FP64 right-hand side and FP64 steps match the oracle to
<= 1e-12 relative (max-norm of the difference over the max-norm of the oracle
field, per variable); the mixed-precision evolution is reported against the
FP64 one as a relative L2 error and must stay <= 1e-6.
"""
import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import CurvedDgEvolution, Shell

pytestmark = pytest.mark.gpu
RTOL = 1e-12
G1, G2 = 0.0, 1.0


def rel_err(a, b):
    """max over vars of ||a_v - b_v||_inf / ||b_v||_inf ([E, 5, N^3] arrays)."""
    a = a.reshape(a.shape[0], 5, -1)
    b = b.reshape(b.shape[0], 5, -1)
    worst = 0.0
    for v in range(5):
        den = np.abs(b[:, v]).max()
        num = np.abs(a[:, v] - b[:, v]).max()
        worst = max(worst, num / den if den > 0 else num)
    return worst


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def make(oracle, ang, rad, n, precision=dgsw.PRECISION_FP64, r_inner=1.9):
    sh = Shell(r_inner, 20.0, ang, rad, "logarithmic", 1.0, G1)
    ev = CurvedDgEvolution(sh, n, precision=precision, gamma2=G2)
    s = oracle.shell(r_inner, 20.0, ang, rad, n, 1.0, G1, G2)
    return ev, s


@pytest.mark.parametrize("ang,rad,n", [(0, 0, 4), (0, 1, 5), (1, 1, 8), (1, 2, 10)])
def test_curved_rhs_random_state_matches_oracle(oracle, ang, rad, n):
    ev, s = make(oracle, ang, rad, n)
    rng = np.random.default_rng(n)
    u = rng.uniform(-1.0, 1.0, ev.state_size)
    ref, ok = oracle.shell_rhs(s, u.reshape(-1, 5, n ** 3))
    assert ok
    got = ev.rhs(u)
    assert rel_err(got.reshape(ref.shape), ref) <= RTOL
    ev.close()


def test_curved_initial_data_matches_oracle(oracle):
    ev, s = make(oracle, 1, 2, 6)
    ev.set_gaussian_shell(1.0, 8.0, 1.0)
    ref = oracle.shell_initial_data(s, 8.0, 1.0)
    np.testing.assert_allclose(ev.get_state().reshape(ref.shape), ref, rtol=0, atol=1e-14)
    ev.close()


def test_curved_steps_match_oracle(oracle):
    n = 6
    ev, s = make(oracle, 1, 1, n)
    ev.set_gaussian_shell(1.0, 8.0, 1.0)
    u0 = ev.get_state()
    ref, ok = oracle.shell_evolve(s, u0.reshape(-1, 5, n ** 3), 1e-2, 10)
    assert ok
    ev.step(10, 1e-2)
    assert rel_err(ev.get_state().reshape(ref.shape), ref) <= 1e-11
    # the same three stages one substep at a time
    ev.set_state(u0)
    for _ in range(10):
        for k in range(3):
            ev.substep(k, 1e-2)
    assert rel_err(ev.get_state().reshape(ref.shape), ref) <= 1e-11
    ev.close()


def test_curved_full_shell_rhs_and_step_match_oracle(oracle):
    # 6 wedges x (4 x 4 x 8) elements, 10 points per dimension, r in [1.9, 20]
    n = 10
    ev, s = make(oracle, 2, 3, n)
    assert ev.n_elements == 768
    ev.set_gaussian_shell(1.0, 8.0, 1.0)
    u0 = ev.get_state()
    ref, ok = oracle.shell_rhs(s, u0.reshape(-1, 5, n ** 3))
    assert ok
    assert rel_err(ev.rhs(u0).reshape(ref.shape), ref) <= RTOL
    ref1, _ = oracle.shell_evolve(s, u0.reshape(-1, 5, n ** 3), 1e-3, 1)
    ev.step(1, 1e-3)
    assert rel_err(ev.get_state().reshape(ref1.shape), ref1) <= RTOL
    ev.close()


def test_curved_excision_outside_horizon_is_rejected(oracle):
    with pytest.raises(dgsw.DgswError, match="DemandOutgoingCharSpeeds"):
        CurvedDgEvolution(Shell(3.0, 20.0, 0, 0), 4, gamma2=G2)


def test_curved_mixed_rhs_close_to_fp64(oracle):
    n = 8
    ev64, s = make(oracle, 1, 2, n)
    evm, _ = make(oracle, 1, 2, n, precision=dgsw.PRECISION_MIXED)
    ev64.set_gaussian_shell(1.0, 8.0, 1.0)
    u = ev64.get_state()
    a = ev64.rhs(u)
    b = evm.rhs(u)
    assert rel_l2(b, a) < 1e-6
    ev64.close()
    evm.close()


def test_curved_mixed_evolution_error(oracle):
    # 200 steps of dt = 1e-3 on the 768-element shell: mixed vs FP64
    n = 10
    ev64, _ = make(oracle, 2, 3, n)
    evm, _ = make(oracle, 2, 3, n, precision=dgsw.PRECISION_MIXED)
    for ev in (ev64, evm):
        ev.set_gaussian_shell(1.0, 8.0, 1.0)
        ev.step(200, 1e-3)
    a, b = ev64.get_state(), evm.get_state()
    assert np.isfinite(b).all()
    err = rel_l2(b, a)
    print("curved mixed vs fp64 relative L2 after 200 steps: %.3e" % err)
    assert err < 1e-6
    ev64.close()
    evm.close()


def test_curved_mixed_n12(oracle):
    # N = 12 on the 768-element shell (the largest extent compiled); two
    # steps against FP64
    n = 12
    ev64, _ = make(oracle, 2, 3, n)
    evm, _ = make(oracle, 2, 3, n, precision=dgsw.PRECISION_MIXED)
    for ev in (ev64, evm):
        ev.set_gaussian_shell(1.0, 8.0, 1.0)
        ev.step(2, 1e-3)
    assert rel_l2(evm.get_state(), ev64.get_state()) < 1e-7
    ev64.close()
    evm.close()


@pytest.mark.parametrize("n", [5, 10, 12])
def test_curved_mixed_launch_shapes_agree(oracle, n):
    # the mixed curved stage kernel's launch shapes (dgsw_tune family
    # mixed_curved: 256 threads at two occupancies, 512 threads; the FP64
    # update fused or as a separate stream): the tuner
    # restores the state it times on, every shape gives the same bits, and
    # all stay within the mixed bar of FP64 over 20 steps
    ev64, _ = make(oracle, 1, 2, n)
    ev64.set_gaussian_shell(1.0, 8.0, 1.0)
    u0 = ev64.get_state()
    ev64.step(20, 1e-3)
    ref = ev64.get_state()
    ev64.close()
    out = []
    evm, _ = make(oracle, 1, 2, n, precision=dgsw.PRECISION_MIXED)
    evm.set_state(u0)
    info = evm.tune()
    assert info["family"] == "mixed_curved"
    assert len(info["ms_per_step"]) == 6
    assert all(ms > 0 for ms in info["ms_per_step"])
    np.testing.assert_array_equal(evm.get_state(), u0)
    for v in range(6):
        assert evm.tune(force_variant=v)["variant"] == v
        evm.set_state(u0)
        evm.step(20, 1e-3)
        out.append(evm.get_state())
    evm.close()
    for got in out:
        assert rel_l2(got, ref) < 1e-6
    for got in out[1:]:
        np.testing.assert_array_equal(out[0], got)
