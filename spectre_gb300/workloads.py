"""Seeded synthetic workloads of the benchmark configurations.

The reference has no benchmark suite for this path; these generators produce
the configurations' shapes, sizes and value distributions from a seed with
numpy's PCG64 generator (numpy.random.default_rng(seed)), so every run (and
the CPU oracle) sees the same instances.
"""
import math

import numpy as np

from .dgsw import Brick

TWO_PI = 2.0 * math.pi


def batched_instances(n_instances=256, seed=2024, counts=(2, 8), points=(4, 10),
                      widths=(0.3, 1.0), amplitudes=(0.5, 2.0)):
    """Independent periodic ScalarWave evolutions on [0, 2pi]^3.

    Per instance: elements per axis uniform in counts (inclusive); per element
    LGL points per dimension uniform in points (inclusive); a Gaussian pulse
    with centre uniform in the cube, width U(widths), amplitude U(amplitudes).
    Returns (bricks, points_per_element int32, params [n_instances, 5] as
    (A, w, cx, cy, cz)).
    """
    rng = np.random.default_rng(seed)
    bricks = []
    for _ in range(n_instances):
        n = rng.integers(counts[0], counts[1] + 1, 3)
        bricks.append(Brick(tuple(int(v) for v in n)))
    n_elem = sum(b.elements[0] * b.elements[1] * b.elements[2] for b in bricks)
    pts = rng.integers(points[0], points[1] + 1, n_elem).astype(np.int32)
    params = np.zeros((n_instances, 5))
    params[:, 0] = rng.uniform(amplitudes[0], amplitudes[1], n_instances)
    params[:, 1] = rng.uniform(widths[0], widths[1], n_instances)
    params[:, 2:5] = rng.uniform(0.0, TWO_PI, (n_instances, 3))
    return bricks, pts, params


def grid_points(points_per_element):
    p = np.asarray(points_per_element, dtype=np.int64)
    return int(np.sum(p ** 3))
