"""Plain FP64 CUDA path vs the CPU FP64 oracle, through the C ABI.

Tolerance: the FP64 right-hand side and each FP64 step must match the oracle
to <= 1e-12 relative (max-norm of the difference over the max-norm of the
oracle field, per variable).
"""
import json
import math
import os

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import STAGE_VARIANTS, Brick, DgEvolution

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
UPW = json.load(open(os.path.join(HERE, "golden", "upwind_golden.json")))
RTOL = 1e-12


def rel_err_per_var(a, b, elem_n):
    """max over vars of ||a_v - b_v||_inf / ||b_v||_inf."""
    off = 0
    worst = 0.0
    num = np.zeros(5)
    den = np.zeros(5)
    for n in elem_n:
        np_ = int(n) ** 3
        for v in range(5):
            sa = a[off + v * np_: off + (v + 1) * np_]
            sb = b[off + v * np_: off + (v + 1) * np_]
            num[v] = max(num[v], np.max(np.abs(sa - sb)))
            den[v] = max(den[v], np.max(np.abs(sb)))
        off += 5 * np_
    for v in range(5):
        if den[v] > 0:
            worst = max(worst, num[v] / den[v])
        else:
            worst = max(worst, num[v])
    return worst


def random_state(rng, bricks, n, oracle):
    size = oracle.offsets(oracle.elem_points(bricks, n))[-1]
    return rng.uniform(-1, 1, int(size))


def test_package_and_boundary_terms_kernels_match_golden(oracle):
    import torch
    dev = "cuda"
    up = dgsw.UpwindPenalty()
    pk = []
    for inp, ref in zip(UPW["inputs"], UPW["packaged"]):
        t = {k: torch.tensor(np.array(v), dtype=torch.float64, device=dev) for k, v in inp.items()}
        p, ms = up.dg_package_data(t["psi"], t["pi"], t["phi"].contiguous(), t["gamma2"],
                                   t["normal"].contiguous())
        np.testing.assert_allclose(p.cpu().numpy(), np.array(ref), rtol=1e-14, atol=1e-15)
        assert ms == 1.0
        pk.append(p)
    bt = up.dg_boundary_terms(pk[0], pk[1]).cpu().numpy()
    np.testing.assert_allclose(bt, np.array(UPW["boundary_terms"]), rtol=1e-14, atol=1e-15)
    sc = UPW["speeds_case"]
    bt2 = up.dg_boundary_terms(torch.tensor(sc["pkg_int"], dtype=torch.float64, device=dev),
                               torch.tensor(sc["pkg_ext"], dtype=torch.float64, device=dev))
    np.testing.assert_allclose(bt2.cpu().numpy(), np.array(sc["boundary_terms"]), rtol=1e-14,
                               atol=1e-15)


def test_package_with_mesh_velocity_matches_oracle(oracle):
    import torch
    rng = np.random.default_rng(11)
    n = 300
    nrm = rng.normal(size=(3, n))
    nrm /= np.linalg.norm(nrm, axis=0)
    args = [rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, (3, n)),
            rng.uniform(0, 2, n), nrm]
    ndv = rng.uniform(-0.5, 0.5, n)
    ref, _ = oracle.package(*args, ndotv=ndv)
    t = [torch.tensor(a, dtype=torch.float64, device="cuda").contiguous() for a in args]
    p, ms = dgsw.UpwindPenalty().dg_package_data(*t, None,
                                                 torch.tensor(ndv, device="cuda"))
    np.testing.assert_allclose(p.cpu().numpy(), ref, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("n", list(range(2, 13)))
def test_rhs_random_state_all_extents(oracle, n):
    rng = np.random.default_rng(100 + n)
    bricks = [Brick((3, 2, 4), (0.0, -1.0, 0.5), (1.5, 2.0, 3.0))]
    u = random_state(rng, bricks, n, oracle)
    ref = oracle.rhs(bricks, n, u)
    with DgEvolution(bricks, n) as ev:
        got = ev.rhs(u)
    assert rel_err_per_var(got, ref, [n] * (len(u) // (5 * n ** 3))) <= RTOL


@pytest.mark.parametrize("gamma2", [0.0, 1.5])
def test_rhs_gamma2_and_multi_instance(oracle, gamma2):
    rng = np.random.default_rng(5)
    bricks = [Brick((2, 3, 2)), Brick((4, 1, 2), (0, 0, 0), (1.0, 2.0, 3.0))]
    n = 5
    u = random_state(rng, bricks, n, oracle)
    ref = oracle.rhs(bricks, n, u, gamma2=gamma2)
    with DgEvolution(bricks, n, gamma2=gamma2) as ev:
        got = ev.rhs(u)
    assert rel_err_per_var(got, ref, [n] * (len(u) // (5 * n ** 3))) <= RTOL


def test_volume_rhs_matches_oracle(oracle):
    import torch
    rng = np.random.default_rng(9)
    bricks = [Brick((2, 2, 2))]
    n = 8
    u = random_state(rng, bricks, n, oracle)
    ref = oracle.rhs(bricks, n, u, volume_only=True)
    with DgEvolution(bricks, n) as ev:
        got = ev.volume_rhs(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel_err_per_var(got, ref, [n] * 8) <= RTOL


def test_config1_rhs_and_substeps(oracle):
    # The plane-wave case: 4^3 elements, N = 6, k = (1,1,1)
    bricks = [Brick((4, 4, 4))]
    n, dt = 6, 1e-3
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    en = [n] * 64
    with DgEvolution(bricks, n) as ev:
        ev.set_initial_data("plane_wave", [1, 1, 1])
        ug = ev.get_state()
        assert rel_err_per_var(ug, u0, en) <= 1e-14
        assert rel_err_per_var(ev.rhs(u0), oracle.rhs(bricks, n, u0), en) <= RTOL
        # substeps one at a time against Rk3HesthavenSsp::update_u
        ev.set_state(u0)
        cur = u0
        for k in range(3):
            ref = oracle.rk3_substep(k, dt, u0, cur, oracle.rhs(bricks, n, cur))
            ev.substep(k, dt)
            got = ev.get_state()
            assert rel_err_per_var(got, ref, en) <= RTOL, k
            cur = ref


def test_config1_full_run_vs_oracle_and_analytic(oracle):
    bricks = [Brick((4, 4, 4))]
    n, dt, steps = 6, 1e-3, 200
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1])
    with DgEvolution(bricks, n) as ev:
        ev.set_state(u0)
        ev.step(1, dt)
        one = ev.get_state()
        ref1 = oracle.evolve(bricks, n, u0, dt, 1)
        assert rel_err_per_var(one, ref1, [n] * 64) <= RTOL
        ev.step(steps - 1, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, n, u0, dt, steps)
    # 200 steps of roundoff-level differences stay far below the per-step bar
    assert rel_err_per_var(got, ref, [n] * 64) <= 200 * RTOL
    ua = oracle.initial_data(bricks, n, "plane_wave", [1, 1, 1], t=dt * steps)
    err = np.max(np.abs(got - ua))
    assert err < 5e-3  # N = 6, 4 elements per 2 pi: discretisation error


def test_graph_chunks_equal_single_steps(oracle):
    bricks = [Brick((2, 2, 2))]
    n, dt = 6, 1e-3
    u0 = oracle.initial_data(bricks, n, "gaussian", oracle.gaussian_params(1, width=1.0))
    with DgEvolution(bricks, n) as ev:
        ev.set_state(u0)
        ev.step(37, dt)            # 2 graphs of 16 steps + 5 single steps
        a = ev.get_state()
        ev.set_state(u0)
        for _ in range(37):
            ev.step(1, dt)
        b = ev.get_state()
    np.testing.assert_array_equal(a, b)


@pytest.mark.slow
def test_config2_full_size_one_step(oracle):
    # The Gaussian-pulse case at full size: 32^3 elements, N = 8, Gaussian pulse, one SSP-RK3
    # step against the oracle (about 16.8M points; the oracle runs multi-threaded).
    bricks = [Brick((32, 32, 32))]
    n, dt = 8, 2e-4
    params = oracle.gaussian_params(1, amp=1.0, width=0.5)
    u0 = oracle.initial_data(bricks, n, "gaussian", params)
    with DgEvolution(bricks, n) as ev:
        ev.set_initial_data("gaussian", params)
        assert rel_err_per_var(ev.get_state(), u0, [n] * 32768) <= 1e-14
        ev.step(1, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, n, u0, dt, 1)
    assert rel_err_per_var(got, ref, [n] * 32768) <= RTOL


def test_linearity_full_size():
    # L(a u + b v) = a L(u) + b L(v) at 32^3 x 8^3, on the device
    import torch
    bricks = [Brick((32, 32, 32))]
    n = 8
    with DgEvolution(bricks, n) as ev:
        g = torch.Generator(device="cuda").manual_seed(3)
        u = torch.rand(ev.state_size, dtype=torch.float64, device="cuda", generator=g)
        v = torch.rand(ev.state_size, dtype=torch.float64, device="cuda", generator=g)
        lu, lv = ev.rhs(u), ev.rhs(v)
        lw = ev.rhs(2.0 * u - 0.5 * v)
        diff = (lw - (2.0 * lu - 0.5 * lv)).abs().max().item()
        scale = lw.abs().max().item()
    assert diff <= 1e-12 * scale


def test_energy_non_increasing():
    # The upwind flux is dissipative: the discrete L2 energy of
    # (Pi^2 + |Phi|^2) does not grow over a step (checked with LGL weights).
    import torch
    bricks = [Brick((4, 4, 4))]
    n = 6
    x, w = dgsw.lgl_points_weights(n)
    W = np.einsum("i,j,k->kji", w, w, w).ravel()
    rng = np.random.default_rng(0)
    with DgEvolution(bricks, n) as ev:
        u = rng.uniform(-1, 1, ev.state_size)
        ev.set_state(u)

        def energy(s):
            s = s.reshape(64, 5, n ** 3)
            return float(np.sum(W * (s[:, 1] ** 2 + s[:, 2] ** 2 + s[:, 3] ** 2 + s[:, 4] ** 2)))

        e0 = energy(u)
        ev.step(5, 2e-3)
        e1 = energy(ev.get_state())
    assert e1 <= e0


def test_errors_are_reported_not_fatal():
    with pytest.raises(dgsw.DgswError) as ei:
        DgEvolution([Brick((2, 2, 2))], 6, precision=7)
    assert ei.value.status == -1
    with DgEvolution([Brick((2, 2, 2))], 4) as ev:
        with pytest.raises(dgsw.DgswError):
            ev.substep(3, 1e-3)
        with pytest.raises(dgsw.DgswError):
            ev.step(-1, 1e-3)
        with pytest.raises(dgsw.DgswError):
            ev.set_initial_data("gaussian", [1.0, -1.0, 0, 0, 0])
        ev.step(1, 1e-3)  # the handle stays usable


def test_autotuned_variants_agree(oracle):
    # every launch configuration of the FP64 stage (two of elements per block,
    # two with the three axis passes at once) matches the oracle, all with
    # the same bits
    bricks = [Brick((3, 2, 4))]
    for n in (2, 4, 5, 8, 10, 11, 12):
        u = random_state(np.random.default_rng(n), bricks, n, oracle)
        ref = oracle.evolve(bricks, n, u, 1e-3, 2)
        first = None
        for force in range(STAGE_VARIANTS):
            with DgEvolution(bricks, n) as ev:
                ev.set_state(u)
                v, ms = ev.autotune(force)
                assert v == force and (ms > 0).all()
                ev.step(2, 1e-3)
                got = ev.get_state()
            assert rel_err_per_var(got, ref, oracle.elem_points(bricks, n)) <= 1e-12
            if first is None:
                first = got
            else:
                assert np.array_equal(got, first), (n, force)
