"""The persistent batch kernels of the mixed-precision path (stage_batch.cu):
elements of any extents in one launch per stage, with exterior face values
passed between stages through compact face buffers.

Checked against the FP64 oracle's SSP-RK3 evolution (rel L2 <= 1e-6 per
instance, the mixed-precision bar), against the per-extent-class mixed path
(DGSW_MIXED_KERNEL=general) and, on uniform meshes (DGSW_MIXED_KERNEL=batch),
for even and odd extents.
"""
import os

import numpy as np
import pytest

from spectre_gb300 import workloads
from spectre_gb300.dgsw import Brick, DgEvolution, PRECISION_MIXED

pytestmark = pytest.mark.gpu
RTOL_MIXED = 1e-6


def instance_slices(bricks, pts):
    out = []
    e = 0
    off = 0
    pts = np.broadcast_to(np.asarray(pts), (sum(b.elements[0] * b.elements[1] * b.elements[2]
                                                for b in bricks),))
    for b in bricks:
        ne = b.elements[0] * b.elements[1] * b.elements[2]
        size = int(5 * np.sum(np.asarray(pts[e:e + ne], dtype=np.int64) ** 3))
        out.append(slice(off, off + size))
        off += size
        e += ne
    return out


def worst_rel_l2(got, ref, bricks, pts):
    return max(float(np.linalg.norm(got[sl] - ref[sl]) / np.linalg.norm(ref[sl]))
               for sl in instance_slices(bricks, pts))


def _evolve(bricks, pts, u0, dt, steps, kernel=None, calls=1):
    old = os.environ.get("DGSW_MIXED_KERNEL")
    if kernel is not None:
        os.environ["DGSW_MIXED_KERNEL"] = kernel
    try:
        with DgEvolution(bricks, pts, precision=PRECISION_MIXED) as ev:
            ev.set_state(u0)
            for _ in range(calls):
                ev.step(steps // calls, dt)
            return ev.get_state()
    finally:
        if old is None:
            os.environ.pop("DGSW_MIXED_KERNEL", None)
        else:
            os.environ["DGSW_MIXED_KERNEL"] = old


@pytest.mark.parametrize("seed", [0, 1])
def test_batch_all_extents_vs_oracle(oracle, seed):
    # every extent 2..12 on two bricks, random per element
    rng = np.random.default_rng(seed)
    bricks = [Brick((3, 2, 2), (0.0, -1.0, 0.5), (1.5, 2.0, 3.0)), Brick((2, 3, 1))]
    E = sum(b.elements[0] * b.elements[1] * b.elements[2] for b in bricks)
    pts = rng.integers(2, 13, E).astype(np.int32)
    params = np.array([[1.0, 0.7, 0.5, 0.0, 1.5], [2.0, 0.9, 3.0, 2.0, 1.0]])
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    dt, steps = 2e-4, 20
    got = _evolve(bricks, pts, u0, dt, steps)
    ref = oracle.evolve(bricks, pts, u0, dt, steps)
    assert worst_rel_l2(got, ref, bricks, pts) <= RTOL_MIXED


def test_batch_matches_class_path_and_survives_split_calls(oracle):
    bricks, pts, params = workloads.batched_instances(8, seed=21)
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    dt, steps = 1e-4, 40
    batch = _evolve(bricks, pts, u0, dt, steps)
    split = _evolve(bricks, pts, u0, dt, steps, calls=4)  # face values re-formed per call
    general = _evolve(bricks, pts, u0, dt, steps, kernel="general")
    ref = oracle.evolve(bricks, pts, u0, dt, steps)
    assert worst_rel_l2(batch, ref, bricks, pts) <= RTOL_MIXED
    assert worst_rel_l2(split, ref, bricks, pts) <= RTOL_MIXED
    assert worst_rel_l2(general, ref, bricks, pts) <= RTOL_MIXED
    assert worst_rel_l2(batch, general, bricks, pts) <= RTOL_MIXED


@pytest.mark.parametrize("n", [5, 6, 8])
def test_batch_uniform_extent_vs_oracle(oracle, n):
    bricks = [Brick((4, 3, 4))]
    u0 = oracle.initial_data(bricks, n, "plane_wave", [1.0, 1.0, 1.0])
    dt, steps = 1e-3, 50
    got = _evolve(bricks, n, u0, dt, steps, kernel="batch")
    ref = oracle.evolve(bricks, n, u0, dt, steps)
    assert worst_rel_l2(got, ref, bricks, [n] * 48) <= RTOL_MIXED


def test_batch_tuner_keeps_state_and_every_shape_agrees(oracle):
    bricks, pts, params = workloads.batched_instances(6, seed=8)
    u0 = oracle.initial_data(bricks, pts, "gaussian", params)
    dt, steps = 1e-4, 10
    ref = oracle.evolve(bricks, pts, u0, dt, steps)
    results = []
    with DgEvolution(bricks, pts, precision=PRECISION_MIXED) as ev:
        ev.set_state(u0)
        info = ev.tune()
        assert info["family"] == "mixed_batch"
        assert np.array_equal(ev.get_state(), u0)  # the timing restores the state
        timed = [v for v, ms in enumerate(info["ms_per_step"]) if ms > 0]
        assert info["variant"] in timed and len(timed) >= 2
        for v in timed:
            assert ev.tune(force_variant=v)["variant"] == v
            ev.set_state(u0)
            ev.step(steps, dt)
            got = ev.get_state()
            assert worst_rel_l2(got, ref, bricks, pts) <= RTOL_MIXED
            results.append(got)
    # every launch shape does the same arithmetic per element
    for r in results[1:]:
        np.testing.assert_array_equal(r, results[0])
