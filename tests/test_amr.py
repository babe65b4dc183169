"""AMR projection of element data (amr::projectors::ProjectVariables,
ParallelAlgorithms/Amr/Projectors/Variables.hpp:25-99), host side.

Pins the oracle to the reference's own known answers
(tests/Unit/ParallelAlgorithms/Amr/Projectors/Test_Variables.cpp): a product
of quadratics in each logical coordinate, p-projected from extent 4 to
extents (3, 4, 5), and h-refined into the lower x half, is reproduced
exactly on the new points.  Then checks the product's host matrices
(dgsw_amr_matrix) against the oracle's for every extent pair and child size,
and the projection identities (truncation after interpolation is the
identity; the half-interval matrices are the refined lattices' ones).
"""
import numpy as np
import pytest

X_COEF = (0.75, -1.75, 2.75)
Y_COEF = (-0.25, 1.25, -2.25)
Z_COEF = (0.125, -1.625, -2.875)


def quad(c, x):
    return c[0] + c[1] * x + c[2] * x * x


def field(oracle, ext, scale, xmap=lambda x: x, dims=3):
    """scale * f(x) f(y) f(z) on LGL points of extents ext (x fastest); the
    factors of the dimensions beyond `dims` are 1 (the reference's 1D / 2D
    cases as blocks of extent 2 there)."""
    xs = [oracle.lgl(n)[0] for n in ext]
    fx = quad(X_COEF, xmap(xs[0]))
    fy = quad(Y_COEF, xs[1]) if dims > 1 else np.ones(ext[1])
    fz = quad(Z_COEF, xs[2]) if dims > 2 else np.ones(ext[2])
    return scale * np.einsum("k,j,i->kji", fz, fy, fx).ravel()


@pytest.mark.parametrize("dims", [1, 2, 3])
def test_oracle_p_refine_known_answer(oracle, dims):
    old = [4, 2 if dims < 2 else 4, 2 if dims < 3 else 4]
    new = [3, 2 if dims < 2 else 4, 2 if dims < 3 else 5]
    u = np.concatenate([field(oracle, old, 1.0, dims=dims), field(oracle, old, 2.0, dims=dims)])
    out, _ = oracle.amr_project(2, [0], [old], [new], [[0, 0, 0]], u, [0])
    want = np.concatenate([field(oracle, new, 1.0, dims=dims), field(oracle, new, 2.0, dims=dims)])
    np.testing.assert_allclose(out, want, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("dims", [1, 2, 3])
def test_oracle_h_refine_known_answer(oracle, dims):
    ext = [4, 2 if dims < 2 else 4, 2 if dims < 3 else 4]
    u = np.concatenate([field(oracle, ext, 1.0, dims=dims), field(oracle, ext, 2.0, dims=dims)])
    out, _ = oracle.amr_project(2, [0], [ext], [ext], [[1, 0, 0]], u, [0])
    lower = lambda x: 0.5 * (x + 1.0) - 1.0  # noqa: E731  child x in the parent's frame
    want = np.concatenate([field(oracle, ext, 1.0, lower, dims),
                           field(oracle, ext, 2.0, lower, dims)])
    np.testing.assert_allclose(out, want, rtol=1e-13, atol=1e-13)


def test_product_matrices_match_oracle(dgsw_lib, oracle):
    worst = 0.0
    for s in range(2, 13):
        for d in range(2, 13):
            for child in (0, 1, 2):
                if child and d < s:
                    with pytest.raises(dgsw_lib.DgswError):
                        dgsw_lib.amr_matrix(s, d, child)
                    continue
                got = dgsw_lib.amr_matrix(s, d, child)
                want = oracle.amr_matrix(s, d, child)
                worst = max(worst, float(np.abs(got - want).max()))
    assert worst <= 2e-13, worst


@pytest.mark.parametrize("n", [2, 4, 7, 12])
def test_projection_identities(dgsw_lib, oracle, n):
    for m in range(n + 1, 13):
        up = dgsw_lib.amr_matrix(n, m, 0)
        down = dgsw_lib.amr_matrix(m, n, 0)
        np.testing.assert_allclose(down @ up, np.eye(n), atol=2e-13)
    for upper in (0, 1):
        P, _ = oracle.proj_half(n, upper)
        np.testing.assert_allclose(dgsw_lib.amr_matrix(n, n, 1 + upper), P, atol=2e-14)


def test_bad_arguments(dgsw_lib):
    for args in ((1, 4, 0), (4, 13, 0), (4, 4, 3), (5, 4, 1)):
        with pytest.raises(dgsw_lib.DgswError):
            dgsw_lib.amr_matrix(*args)
