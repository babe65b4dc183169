"""AMR projection of element data on the device (dgsw_amr_project_device)
against the oracle's ProjectVariables, and the reference's known answers
(Test_Variables.cpp: p-projection 4 -> (3, 4, 5) and h-refinement into the
lower x half of a product of quadratics are exact)."""
import numpy as np
import pytest

from tests.test_amr import field

pytestmark = pytest.mark.gpu


def _owner():
    from spectre_gb300 import Brick, DgEvolution
    return DgEvolution([Brick((1, 1, 1))], 4, device=0)


def test_known_answers_on_device(oracle):
    import torch
    from spectre_gb300.dgsw import amr_project
    old, new = [4, 4, 4], [3, 4, 5]
    u = np.concatenate([field(oracle, old, 1.0), field(oracle, old, 2.0)])
    with _owner() as ev:
        t = torch.from_numpy(u).cuda()
        out, _ = amr_project(ev, 2, t, [0], [0, 0], [old, old], [new, old], [[0, 0, 0], [1, 0, 0]])
        got = out.cpu().numpy()
    lower = lambda x: 0.5 * (x + 1.0) - 1.0  # noqa: E731
    want = np.concatenate([field(oracle, new, 1.0), field(oracle, new, 2.0),
                           field(oracle, old, 1.0, lower), field(oracle, old, 2.0, lower)])
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_maps_match_oracle(oracle, seed):
    import torch
    from spectre_gb300.dgsw import amr_project
    rng = np.random.default_rng(seed)
    n_in, n_out, n_vars = 40, 200, 5
    in_ext = rng.integers(2, 13, size=(n_in, 3))
    sizes = n_vars * np.prod(in_ext, axis=1)
    in_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    u = rng.standard_normal(int(sizes.sum()))
    src = rng.integers(0, n_in, size=n_out).astype(np.int32)
    se = in_ext[src]
    child = rng.integers(0, 3, size=(n_out, 3))
    de = np.where(child > 0, rng.integers(se, 13), rng.integers(2, 13, size=(n_out, 3)))
    with _owner() as ev:
        out, off = amr_project(ev, n_vars, torch.from_numpy(u).cuda(), in_off, src, se, de, child)
        got = out.cpu().numpy()
    want, off_o = oracle.amr_project(n_vars, src, se, de, child, u, in_off)
    np.testing.assert_array_equal(off, off_o)
    scale = np.abs(u).max()
    assert float(np.abs(got - want).max()) <= 1e-12 * scale


def test_h_refined_state_is_exact_for_polynomials(oracle):
    """Every element of a 2^3 brick of N = 6 holding a degree-5 polynomial in x
    refined into its 8 children reproduces the polynomial on the children's
    points."""
    import torch
    from spectre_gb300.dgsw import amr_project
    n = 6
    x, _ = oracle.lgl(n)
    poly = lambda t: 0.3 - 1.1 * t + 0.7 * t ** 3 - 0.2 * t ** 5  # noqa: E731
    blk = np.tile(np.einsum("k,j,i->kji", np.ones(n), np.ones(n), poly(x)).ravel(), 5)
    u = np.tile(blk, 8)
    in_off = np.arange(8, dtype=np.int64) * blk.size
    src, child = [], []
    for e in range(8):
        for c in range(8):
            src.append(e)
            child.append([1 + (c & 1), 1 + ((c >> 1) & 1), 1 + ((c >> 2) & 1)])
    ext = [[n, n, n]] * len(src)
    with _owner() as ev:
        out, _ = amr_project(ev, 5, torch.from_numpy(u).cuda(), in_off, src, ext, ext, child)
        got = out.cpu().numpy().reshape(len(src), 5, n, n, n)
    for k, ch in enumerate(child):
        s = 1.0 if ch[0] == 2 else -1.0
        want = poly(0.5 * (x + s))
        np.testing.assert_allclose(got[k], np.broadcast_to(want, (5, n, n, n)), atol=1e-13)


def test_refuses_bad_maps():
    import torch
    from spectre_gb300.dgsw import DgswError, amr_project
    u = torch.zeros(5 * 64, dtype=torch.float64, device="cuda")
    with _owner() as ev:
        with pytest.raises(DgswError):   # half interval to a coarser extent
            amr_project(ev, 5, u, [0], [0], [[4, 4, 4]], [[3, 4, 4]], [[1, 0, 0]])
        with pytest.raises(DgswError):   # source index out of range
            amr_project(ev, 5, u, [0], [1], [[4, 4, 4]], [[4, 4, 4]], [[0, 0, 0]])
