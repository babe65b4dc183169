"""Batched evolutions with per-element LGL extents (p-nonconforming mortars):
the general CUDA path against the FP64 oracle, and mixed against FP64.

Tolerances as for the uniform path: FP64 right-hand side and steps <= 1e-12
relative (max-norm per variable); mixed vs FP64 <= 1e-6 relative L2 per
instance.
"""
import numpy as np
import pytest

from spectre_gb300 import workloads
from spectre_gb300.dgsw import Brick, DgEvolution, PRECISION_FP64, PRECISION_MIXED

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def per_var_rel(a, b, pts):
    num = np.zeros(5)
    den = np.zeros(5)
    off = 0
    for n in pts:
        np_ = int(n) ** 3
        A = a[off:off + 5 * np_].reshape(5, np_)
        B = b[off:off + 5 * np_].reshape(5, np_)
        num = np.maximum(num, np.max(np.abs(A - B), axis=1))
        den = np.maximum(den, np.max(np.abs(B), axis=1))
        off += 5 * np_
    return float(np.max(num / np.where(den > 0, den, 1.0)))


def instance_slices(bricks, pts):
    out = []
    e = 0
    off = 0
    for b in bricks:
        ne = b.elements[0] * b.elements[1] * b.elements[2]
        size = int(5 * np.sum(np.asarray(pts[e:e + ne], dtype=np.int64) ** 3))
        out.append(slice(off, off + size))
        off += size
        e += ne
    return out


def random_pts(rng, bricks, lo, hi):
    E = sum(b.elements[0] * b.elements[1] * b.elements[2] for b in bricks)
    return rng.integers(lo, hi + 1, E).astype(np.int32)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_general_rhs_random_extents(oracle, seed):
    rng = np.random.default_rng(seed)
    bricks = [Brick((3, 2, 2), (0.0, -1.0, 0.5), (1.5, 2.0, 3.0)), Brick((2, 5, 1))]
    pts = random_pts(rng, bricks, 2, 12)
    size = int(oracle.offsets(pts)[-1])
    u = rng.uniform(-1, 1, size)
    ref = oracle.rhs(bricks, pts, u)
    with DgEvolution(bricks, pts) as ev:
        got = ev.rhs(u)
    assert per_var_rel(got, ref, pts) <= RTOL


def test_general_rhs_gamma2_and_volume(oracle):
    import torch
    rng = np.random.default_rng(7)
    bricks = [Brick((2, 3, 2))]
    pts = random_pts(rng, bricks, 3, 9)
    size = int(oracle.offsets(pts)[-1])
    u = rng.uniform(-1, 1, size)
    ref = oracle.rhs(bricks, pts, u, gamma2=0.7)
    with DgEvolution(bricks, pts, gamma2=0.7) as ev:
        got = ev.rhs(u)
        vol = ev.volume_rhs(torch.tensor(u, device="cuda")).cpu().numpy()
    assert per_var_rel(got, ref, pts) <= RTOL
    assert per_var_rel(vol, oracle.rhs(bricks, pts, u, gamma2=0.7, volume_only=True), pts) <= RTOL


def test_general_substeps(oracle):
    rng = np.random.default_rng(11)
    bricks = [Brick((2, 2, 3))]
    pts = random_pts(rng, bricks, 4, 10)
    params = np.array([[1.3, 0.6, 1.0, 2.0, 3.0]])
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    dt = 1e-3
    with DgEvolution(bricks, pts) as ev:
        ev.set_state(u0)
        cur = u0
        for k in range(3):
            ref = oracle.rk3_substep(k, dt, u0, cur, oracle.rhs(bricks, pts, cur))
            ev.substep(k, dt)
            got = ev.get_state()
            assert per_var_rel(got, ref, pts) <= RTOL, k
            cur = ref


def test_batched_evolution_matches_oracle(oracle):
    # 12 instances drawn like the 256-instance batch, 10 SSP-RK3 steps at dt = 1e-4
    bricks, pts, params = workloads.batched_instances(12, seed=5)
    dt, steps = 1e-4, 10
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    with DgEvolution(bricks, pts) as ev:
        ev.set_initial_data("gaussian", params)
        assert per_var_rel(ev.get_state(), u0, pts) <= 1e-14
        ev.step(steps, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, pts, u0, dt, steps)
    assert per_var_rel(got, ref, pts) <= 10 * RTOL


def first_instances(k, n_instances=256, seed=2024):
    """The first k instances of the seeded 256-instance batch, exactly as they
    appear in it (the generator draws every instance's element counts first,
    then every element's extent, then the pulses)."""
    bricks, pts, params = workloads.batched_instances(n_instances, seed=seed)
    ne = sum(b.elements[0] * b.elements[1] * b.elements[2] for b in bricks[:k])
    return bricks[:k], pts[:ne], params[:k]


@pytest.mark.slow
def test_batched_mixed_vs_oracle_per_instance(oracle):
    # 12 instances of the 256-instance batch over the configured 300 steps at
    # dt = 1e-4: mixed against the FP64 oracle, rel L2 per instance
    bricks, pts, params = first_instances(12)
    dt, steps = 1e-4, 300
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    with DgEvolution(bricks, pts, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        ev.step(steps, dt)
        got = ev.get_state()
    ref = oracle.evolve(bricks, pts, u0, dt, steps)
    for sl in instance_slices(bricks, pts):
        err = np.linalg.norm(got[sl] - ref[sl]) / np.linalg.norm(ref[sl])
        assert err <= 1e-6, err


def test_batched_mixed_rhs(oracle):
    rng = np.random.default_rng(3)
    bricks = [Brick((2, 3, 2)), Brick((3, 1, 2))]
    pts = random_pts(rng, bricks, 2, 12)
    params = np.array([[1.0, 0.7, 0.5, 1.0, 1.5], [2.0, 0.9, 3.0, 2.0, 1.0]])
    u = oracle.initial_data(bricks, pts, "gaussian", params)
    u += 0.05 * rng.uniform(-1, 1, u.size)
    ref = oracle.rhs(bricks, pts, u)
    with DgEvolution(bricks, pts, precision=PRECISION_MIXED) as ev:
        got = ev.rhs(u)
    assert per_var_rel(got, ref, pts) <= 1e-6


@pytest.mark.slow
def test_config3_full_size(oracle):
    # The 256-instance batch at full size; one FP64 step against the oracle,
    # then the configured 300 steps mixed vs FP64 on the device, rel L2 per
    # instance for every instance
    bricks, pts, params = workloads.batched_instances(256, seed=2024)
    dt = 1e-4
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    with DgEvolution(bricks, pts) as a:
        a.set_state(u0)
        a.step(1, dt)
        one = a.get_state()
        ref1 = oracle.evolve(bricks, pts, u0, dt, 1)
        assert per_var_rel(one, ref1, pts) <= RTOL
        a.step(299, dt)
        ua = a.get_state()
    with DgEvolution(bricks, pts, precision=PRECISION_MIXED) as b:
        b.set_state(u0)
        b.step(300, dt)
        ub = b.get_state()
    worst = 0.0
    for sl in instance_slices(bricks, pts):
        worst = max(worst, np.linalg.norm(ub[sl] - ua[sl]) / np.linalg.norm(ua[sl]))
    assert worst <= 1e-6, worst
