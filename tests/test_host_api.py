"""Host-only parts of libdgsw.so (no GPU): exports, spectral setup, index maps,
argument validation."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from spectre_gb300 import dgsw
from spectre_gb300.dgsw import Brick

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LGL = json.load(open(os.path.join(HERE, "golden", "lgl_golden.json")))


def header_functions():
    src = open(os.path.join(ROOT, "include", "dgsw.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dgsw_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol(dgsw_lib):
    names = header_functions()
    assert len(names) >= 20
    L = dgsw_lib.lib()
    for n in names:
        assert hasattr(L, n), n
    # the Python binding declares a signature for every exported function
    assert set(names) <= set(dgsw.exported_symbols()) | {"dgsw_stream"}
    assert L.dgsw_abi_version() == 9


@pytest.mark.parametrize("n", sorted(int(k) for k in LGL["points_weights"]))
def test_product_lgl_matches_golden(dgsw_lib, oracle, n):
    x, w = dgsw.lgl_points_weights(n)
    g = LGL["points_weights"][str(n)]
    np.testing.assert_allclose(x, g["x"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(w, g["w"], rtol=1e-8, atol=1e-8)
    xo, wo = oracle.lgl(n)
    np.testing.assert_allclose(x, xo, rtol=0, atol=4e-16)
    np.testing.assert_allclose(w, wo, rtol=1e-14)


@pytest.mark.parametrize("n", range(2, 21))
def test_product_diff_matrix_matches_oracle(dgsw_lib, oracle, n):
    D = dgsw.differentiation_matrix(n)
    np.testing.assert_allclose(D, oracle.diff_matrix(n), rtol=1e-13, atol=1e-12)
    if str(n) in LGL["diff_matrix"]:
        np.testing.assert_allclose(D, np.array(LGL["diff_matrix"][str(n)]), rtol=1e-13,
                                   atol=1e-13)


def test_product_mortar_projections_match_oracle(dgsw_lib, oracle):
    for ne in range(2, 13):
        for nm in range(ne, 13):
            a, b = dgsw.mortar_projections(ne, nm)
            np.testing.assert_allclose(a, oracle.proj_face_to_mortar(ne, nm), atol=1e-14)
            np.testing.assert_allclose(b, oracle.proj_mortar_to_face(ne, nm), atol=2e-13)


CASES = [
    [Brick((4, 4, 4))],                     # the 4^3 plane-wave lattice
    [Brick((32, 32, 32))],                  # the 32^3 lattice (32,768 elements)
    [Brick((8, 8, 8))],                     # the 8^3 adjoint lattice
    [Brick((3, 6, 5)), Brick((2, 7, 8)), Brick((1, 1, 1))],
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_index_maps_bit_exact(dgsw_lib, oracle, case):
    bricks = CASES[case]
    ids, nbr, mort, fits = dgsw.index_maps(bricks, 6)
    oids, onbr, _, _, ofits = oracle.index_maps(bricks)
    assert fits == ofits
    np.testing.assert_array_equal(ids, oids)
    np.testing.assert_array_equal(nbr, onbr)
    assert (mort == 6).all()


def test_index_maps_random_batched(dgsw_lib, oracle):
    # batches like the 256-instance one: per-axis counts in {2..8}, per-element N in {4..10}
    rng = np.random.default_rng(7)
    bricks = [Brick(tuple(int(v) for v in rng.integers(2, 9, 3))) for _ in range(24)]
    E = oracle.num_elements(bricks)
    pts = rng.integers(4, 11, E).astype(np.int32)
    ids, nbr, mort, fits = dgsw.index_maps(bricks, pts)
    oids, onbr, _, _, ofits = oracle.index_maps(bricks)
    assert fits == ofits
    np.testing.assert_array_equal(ids, oids)
    np.testing.assert_array_equal(nbr, onbr)
    np.testing.assert_array_equal(mort, np.maximum(pts[:, None], pts[onbr]))


def test_index_maps_block_id_overflow(dgsw_lib, oracle):
    # 7x7x7 odd counts need 343 blocks: more than the 8 block-id bits hold
    ids, nbr, mort, fits = dgsw.index_maps([Brick((7, 7, 7))], 4)
    assert not fits
    _, onbr, _, _, ofits = oracle.index_maps([Brick((7, 7, 7))])
    assert not ofits
    np.testing.assert_array_equal(nbr, onbr)


@pytest.mark.parametrize("bad", [
    dict(bricks=[Brick((0, 1, 1))], points=4),
    dict(bricks=[Brick((1, 1, 1), (0, 0, 0), (0, 1, 1))], points=4),
    dict(bricks=[Brick((2, 2, 2))], points=1),
    dict(bricks=[Brick((2, 2, 2))], points=13),
    dict(bricks=[Brick((5000, 1, 1))], points=4),
])
def test_bad_configs_rejected(dgsw_lib, bad):
    with pytest.raises(dgsw.DgswError) as ei:
        dgsw.index_maps(bad["bricks"], bad["points"])
    assert ei.value.status == -1


def test_bad_spectral_arguments(dgsw_lib):
    L = dgsw_lib.lib()
    x = np.zeros(40)
    assert L.dgsw_lgl_points_weights(1, x.ctypes.data, x.ctypes.data) == -1
    assert L.dgsw_lgl_points_weights(21, x.ctypes.data, x.ctypes.data) == -1
    assert L.dgsw_differentiation_matrix(0, x.ctypes.data) == -1
    assert L.dgsw_mortar_projections(5, 4, None, None) == -1
    assert b"ne <= nm" in L.dgsw_last_error(None)


def test_null_handle_is_an_error_not_a_crash(dgsw_lib):
    L = dgsw_lib.lib()
    assert L.dgsw_step(None, 1, 1e-3) == -1
    assert L.dgsw_rhs(None, None, None) == -1
    assert L.dgsw_destroy(None) == 0
    assert L.dgsw_create(None, None) == -1


def test_adams_configs_rejected_before_any_device_work(dgsw_lib):
    # bad AdamsBashforth requests fail with their own status, with or
    # without a GPU (a valid request here reaches the device check)
    import ctypes
    L = dgsw_lib.lib()
    E = 4 * 4 * 4

    def create(levels=None, order=3, precision=dgsw.PRECISION_FP64, points=4):
        holder = dgsw._ConfigHolder([dgsw.Brick((4, 4, 4))], points, precision=precision,
                                    time_stepper="adams_bashforth", order=order,
                                    step_levels=levels)
        h = ctypes.c_void_p()
        return L.dgsw_create(ctypes.byref(holder.cfg), ctypes.byref(h)), h

    rc, _ = create(levels=np.full(E, 4, np.int32))
    assert rc == -1 and b"step levels" in L.dgsw_last_error(None)
    rc, _ = create(order=9)
    assert rc == -1 and b"order" in L.dgsw_last_error(None)
    rc, _ = create(precision=dgsw.PRECISION_MIXED)
    assert rc == -3
    for ok in (dict(levels=np.zeros(E, np.int32)),
               # per-element extents (p-nonconforming faces) are accepted too
               dict(points=np.full(E, 4, np.int32).tolist()[:-1] + [5])):
        rc, h = create(**ok)
        assert rc in (0, -5)  # ok with a GPU, no device without one
        if rc == 0:
            L.dgsw_destroy(h)


def test_double_float_configs_checked_before_any_device_work(dgsw_lib):
    # double-float precision: flat, one extent, SSP-RK3; other requests fail
    # as unsupported, with or without a GPU
    import ctypes
    L = dgsw_lib.lib()
    E = 2 * 2 * 2

    def create(points=4, **kw):
        holder = dgsw._ConfigHolder([dgsw.Brick((2, 2, 2))], points,
                                    precision=dgsw.PRECISION_DOUBLE_FLOAT, **kw)
        h = ctypes.c_void_p()
        return L.dgsw_create(ctypes.byref(holder.cfg), ctypes.byref(h)), h

    for bad in (dict(points=[4] * (E - 1) + [5]), dict(time_stepper="adams_bashforth")):
        rc, _ = create(**bad)
        assert rc == -3 and b"double-float" in L.dgsw_last_error(None), bad
    for ok in (dict(), dict(gamma2=1.5)):
        rc, h = create(**ok)
        assert rc in (0, -5)  # ok with a GPU, no device without one
        if rc == 0:
            L.dgsw_destroy(h)


# ---------------- curved shell: maps and geometry against the oracle ----------------

SHELLS = [dict(ref_ang=0, ref_rad=0, n=4), dict(ref_ang=1, ref_rad=2, n=5),
          dict(ref_ang=2, ref_rad=3, n=10)]


@pytest.mark.parametrize("case", range(len(SHELLS)))
def test_shell_maps_bit_exact(dgsw_lib, oracle, case):
    c = SHELLS[case]
    shell = dgsw.Shell(1.9, 20.0, c["ref_ang"], c["ref_rad"])
    s = oracle.shell(1.9, 20.0, c["ref_ang"], c["ref_rad"], c["n"])
    ids, nbr, mort, fits = dgsw.index_maps(shell, c["n"])
    onbr, operm, oids = oracle.shell_connectivity(s)
    assert fits
    assert ids.tolist() == oids.tolist()
    assert (nbr == onbr).all()
    assert ((mort == 0) == (nbr < 0)).all() and (mort[nbr >= 0] == c["n"]).all()
    xyz, ij, perm = dgsw.shell_geometry(shell, c["n"])
    assert (perm[nbr >= 0] == operm[nbr >= 0]).all()
    oxyz, oij = oracle.shell_geometry(s)
    np.testing.assert_allclose(xyz, oxyz, rtol=0, atol=1e-13 * 20)
    scale = np.abs(oij).max()
    np.testing.assert_allclose(ij, oij, rtol=0, atol=1e-13 * scale)
    # element counts of the reference's Sphere (shell) domain
    assert len(ids) == 6 * 4 ** c["ref_ang"] * 2 ** c["ref_rad"]


@pytest.mark.parametrize("bad", [
    dict(inner_radius=0.0), dict(inner_radius=5.0, outer_radius=4.0),
    dict(refinement_angular=-1), dict(radial_distribution="cubic"), dict(mass=-1.0),
])
def test_bad_shells_rejected(dgsw_lib, bad):
    args = dict(inner_radius=1.9, outer_radius=20.0, refinement_angular=0, refinement_radial=0,
                radial_distribution="logarithmic", mass=1.0)
    if bad.get("radial_distribution") == "cubic":
        with pytest.raises(KeyError):
            dgsw.index_maps(dgsw.Shell(**{**args, **bad}), 4)
        return
    with pytest.raises(dgsw.DgswError):
        dgsw.index_maps(dgsw.Shell(**{**args, **bad}), 4)
