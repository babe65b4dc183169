"""ctypes binding of oracle/_build/liboracle.so (test infrastructure only).

The library is the C++ FP64 restatement in dgsw_oracle.cpp; see its header for
the reference file:line each function follows.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the same sources built for speed (FMA contraction, the host CPU's vector
# ISA): used only as the timed CPU baseline, never as the checker
LIB_FAST = os.path.join(HERE, "_build", "liboracle_fast.so")


class OrcBrick(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
                ("n", ctypes.c_int32 * 3)]


class OrcRefinedBrick(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
                ("blocks", ctypes.c_int32 * 3), ("level", ctypes.c_void_p)]


class OrcShell(ctypes.Structure):
    _fields_ = [("r_inner", ctypes.c_double), ("r_outer", ctypes.c_double),
                ("ref_ang", ctypes.c_int32), ("ref_rad", ctypes.c_int32),
                ("n", ctypes.c_int32), ("mass", ctypes.c_double),
                ("gamma1", ctypes.c_double), ("gamma2", ctypes.c_double)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None
_lib_fast = None


def fast_build_flags():
    """The compiler flags of liboracle_fast.so on this host."""
    r = subprocess.run(["make", "-s", "-C", HERE, "flags"], check=True, capture_output=True,
                       text=True)
    return r.stdout.strip()


def lib(fast=False):
    """The checker library, or with fast=True the speed build of the same
    sources (the timed CPU baseline)."""
    global _lib, _lib_fast
    if fast:
        if _lib_fast is None:
            _lib_fast = _load(LIB_FAST)
        return _lib_fast
    if _lib is None:
        _lib = _load(LIB)
    return _lib


def _load(path):
    srcs = ("dgsw_oracle.cpp", "adams_oracle.cpp", "dgsw_oracle.h", "adams_oracle.hpp")
    if not os.path.exists(path) or os.path.getmtime(path) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in srcs):
        build()
    L = ctypes.CDLL(path)
    P, D, I, I64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64
    sig = {
        "orc_lgl": [I, P, P], "orc_barycentric_weights": [I, P],
        "orc_diff_matrix": [I, P], "orc_vandermonde": [I, P],
        "orc_inv_vandermonde": [I, P], "orc_interp_matrix": [I, I, P, P],
        "orc_proj_face_to_mortar": [I, I, P], "orc_proj_mortar_to_face": [I, I, P],
        "orc_index_maps": [I, P, P, P, P, P], "orc_offsets": [I64, P, P],
        "orc_coords": [I, P, P, P], "orc_initial_data": [I, P, P, I, P, D, P],
        "orc_package": [I, P, P, P, P, P, P, P, P], "orc_boundary_terms": [I, P, P, P],
        "orc_rhs": [I, P, P, D, P, P, I], "orc_volume_rhs": [I, P, P, D, P, P, I],
        "orc_rk3_substep": [I64, I, D, P, P, P, P], "orc_evolve": [I, P, P, D, D, I, P, I],
        "orc_ks_background": [I, D, P, P],
        "orc_csw_time_derivative": [I, P, P, P, P, P, P, D, D, P],
        "orc_csw_package": [I, P, P, P, P, P, P, P, P, P, P, P, P],
        "orc_csw_boundary_terms": [I, P, P, P],
        "orc_csw_cpsr": [I] + [P] * 17,
        "orc_shell_geometry": [P, P, P], "orc_shell_connectivity": [P, P, P, P],
        "orc_shell_initial_data": [P, D, D, P], "orc_shell_rhs": [P, P, P, I],
        "orc_shell_evolve": [P, D, I, P, I],
        "orc_exponential_filter": [I, D, I, P], "orc_filter_elements": [I64, P, D, I, P],
        "orc_observe_norms": [I, P, P, P, P, P], "orc_shell_observe_norms": [P, P, P],
        "orc_lg": [I, P, P], "orc_lg_diff_matrix": [I, P], "orc_lg_boundary": [I, P, P, P, P],
        "orc_coords_gauss": [I, P, I, P], "orc_rhs_gauss": [I, P, I, D, P, P, I],
        "orc_evolve_gauss": [I, P, I, D, D, I, P, I],
        "orc_refined_index_maps": [P, P, P, P], "orc_refined_coords": [P, I, P],
        "orc_refined_rhs": [P, I, D, P, P, I], "orc_refined_evolve": [P, I, D, D, I, P, I],
        "orc_proj_half": [I, I, P, P],
        "orc_amr_matrix": [I, I, I, P], "orc_amr_project": [I, I64, P, P, P, P, P, P, P, P],
        "orc_variable_coefficients": [I, P, D, D, P],
        "orc_adams_coefficients": [I, P, I64, I64, D, I64, P],
        "orc_lts_coefficients": [I, P, P, I, P, P, I64, I64, D, I64, I, I, I, I, P, P, P],
        "orc_evolve_adams": [I, P, I, D, I, P, D, I, P, I],
        "orc_evolve_adams_extents": [I, P, P, D, I, P, D, I, P, I],
        "orc_shell_evolve_adams": [P, I, P, D, I, P, I],
        "orc_shell_evolve_adams_filtered": [P, I, P, D, I, D, I, P, I],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = I
    L.orc_num_elements.argtypes = [I, P]
    L.orc_num_elements.restype = I64
    L.orc_refined_num_elements.argtypes = [P]
    L.orc_refined_num_elements.restype = I64
    L.orc_shell_num_elements.argtypes = [P]
    L.orc_shell_num_elements.restype = I64
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def _bricks(bricks):
    arr = (OrcBrick * len(bricks))()
    for i, b in enumerate(bricks):
        arr[i].lo[:] = [float(v) for v in b.lower]
        arr[i].hi[:] = [float(v) for v in b.upper]
        arr[i].n[:] = [int(v) for v in b.elements]
    return arr


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle call failed with %d" % rc)


def lgl(n):
    x, w = np.zeros(n), np.zeros(n)
    _check(lib().orc_lgl(n, _p(x), _p(w)))
    return x, w


def diff_matrix(n):
    D = np.zeros((n, n))
    _check(lib().orc_diff_matrix(n, _p(D)))
    return D


def vandermonde(n):
    V = np.zeros((n, n))
    _check(lib().orc_vandermonde(n, _p(V)))
    return V


def inv_vandermonde(n):
    V = np.zeros((n, n))
    _check(lib().orc_inv_vandermonde(n, _p(V)))
    return V


def proj_face_to_mortar(ne, nm):
    P = np.zeros((nm, ne))
    _check(lib().orc_proj_face_to_mortar(ne, nm, _p(P)))
    return P


def proj_mortar_to_face(ne, nm):
    P = np.zeros((ne, nm))
    _check(lib().orc_proj_mortar_to_face(ne, nm, _p(P)))
    return P


def num_elements(bricks):
    arr = _bricks(bricks)
    return lib().orc_num_elements(len(bricks), ctypes.addressof(arr))


def index_maps(bricks):
    arr = _bricks(bricks)
    E = lib().orc_num_elements(len(bricks), ctypes.addressof(arr))
    ids = np.zeros(E, dtype=np.uint64)
    nbr = np.zeros((E, 6), dtype=np.int32)
    ijk = np.zeros((E, 3), dtype=np.int32)
    inst = np.zeros(E, dtype=np.int32)
    rc = lib().orc_index_maps(len(bricks), ctypes.addressof(arr), _p(ids), _p(nbr), _p(ijk),
                              _p(inst))
    if rc not in (0, -2):
        _check(rc)
    return ids, nbr, ijk, inst, rc == 0


def offsets(elem_n):
    elem_n = np.ascontiguousarray(elem_n, dtype=np.int32)
    off = np.zeros(len(elem_n) + 1, dtype=np.int64)
    _check(lib().orc_offsets(len(elem_n), _p(elem_n), _p(off)))
    return off


def elem_points(bricks, points):
    E = num_elements(bricks)
    if np.ndim(points) == 0:
        return np.full(E, int(points), dtype=np.int32)
    return np.ascontiguousarray(points, dtype=np.int32)


def coords(bricks, points):
    en = elem_points(bricks, points)
    off = offsets(en)
    xyz = np.zeros(3 * int(off[-1]) // 5)
    arr = _bricks(bricks)
    _check(lib().orc_coords(len(bricks), ctypes.addressof(arr), _p(en), _p(xyz)))
    return xyz


def initial_data(bricks, points, kind, params, t=0.0):
    en = elem_points(bricks, points)
    off = offsets(en)
    u = np.zeros(int(off[-1]))
    p = np.ascontiguousarray(params, dtype=np.float64).ravel()
    arr = _bricks(bricks)
    k = {"plane_wave": 0, "gaussian": 1}[kind]
    _check(lib().orc_initial_data(len(bricks), ctypes.addressof(arr), _p(en), k, _p(p), t, _p(u)))
    return u


def package(psi, pi, phi, gamma2, normal, ndotv=None):
    n = len(psi)
    out = np.zeros((16, n))
    ms = ctypes.c_double()
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (psi, pi, phi, gamma2, normal)]
    nd = None if ndotv is None else np.ascontiguousarray(ndotv, dtype=np.float64)
    _check(lib().orc_package(n, *[_p(a) for a in args], _p(nd), _p(out),
                             ctypes.addressof(ms)))
    return out, ms.value


def boundary_terms(pkg_int, pkg_ext):
    n = pkg_int.shape[1]
    out = np.zeros((5, n))
    a = np.ascontiguousarray(pkg_int, dtype=np.float64)
    b = np.ascontiguousarray(pkg_ext, dtype=np.float64)
    _check(lib().orc_boundary_terms(n, _p(a), _p(b), _p(out)))
    return out


def rhs(bricks, points, u, gamma2=0.0, threads=0, volume_only=False):
    en = elem_points(bricks, points)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros_like(u)
    arr = _bricks(bricks)
    fn = lib().orc_volume_rhs if volume_only else lib().orc_rhs
    _check(fn(len(bricks), ctypes.addressof(arr), _p(en), gamma2, _p(u), _p(out), threads))
    return out


def rk3_substep(k, dt, u0, ucur, dudt):
    out = np.zeros_like(u0)
    _check(lib().orc_rk3_substep(len(u0), k, dt, _p(u0), _p(ucur), _p(dudt), _p(out)))
    return out


def evolve(bricks, points, u, dt, steps, gamma2=0.0, threads=0, fast=False):
    en = elem_points(bricks, points)
    u = np.array(u, dtype=np.float64, copy=True)
    arr = _bricks(bricks)
    _check(lib(fast).orc_evolve(len(bricks), ctypes.addressof(arr), _p(en), gamma2, dt, steps,
                            _p(u), threads))
    return u


def gaussian_params(n_inst, amp=1.0, width=0.5, center=(math.pi, math.pi, math.pi)):
    return np.tile(np.array([amp, width, *center], dtype=np.float64), (n_inst, 1))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def ks_background(xyz, mass=1.0):
    """26 x npts: lapse, shift[3], d_lapse[3], d_shift[9] (d_i shift^j),
    inverse metric[6], trace Christoffel[3], trace K."""
    xyz = _c(xyz)
    n = xyz.shape[1]
    bg = np.zeros((26, n))
    _check(lib().orc_ks_background(n, mass, _p(xyz), _p(bg)))
    return bg


def csw_time_derivative(d_psi, d_pi, d_phi, pi, phi, bg, gamma1, gamma2):
    d_psi, d_pi, d_phi, pi, phi, bg = map(_c, (d_psi, d_pi, d_phi, pi, phi, bg))
    n = pi.shape[0]
    dt = np.zeros((5, n))
    _check(lib().orc_csw_time_derivative(n, _p(d_psi), _p(d_pi), _p(d_phi), _p(pi), _p(phi),
                                         _p(bg), gamma1, gamma2, _p(dt)))
    return dt


def csw_package(psi, pi, phi, lapse, shift, gamma1, gamma2, normal, normal_vector, ndotv=None):
    a = [_c(x) for x in (psi, pi, phi, lapse, shift, gamma1, gamma2, normal, normal_vector)]
    n = a[0].shape[0]
    out = np.zeros((14, n))
    ms = ctypes.c_double()
    nd = None if ndotv is None else _c(ndotv)
    _check(lib().orc_csw_package(n, *[_p(x) for x in a], _p(nd), _p(out), ctypes.addressof(ms)))
    return out, ms.value


def csw_boundary_terms(pkg_int, pkg_ext):
    a, b = _c(pkg_int), _c(pkg_ext)
    out = np.zeros((5, a.shape[1]))
    _check(lib().orc_csw_boundary_terms(a.shape[1], _p(a), _p(b), _p(out)))
    return out


def csw_cpsr(psi, pi, phi, lapse, shift, gamma1, gamma2, normal, normal_vector, xyz, d_psi,
             d_pi, d_phi, dt_psi, dt_pi, dt_phi):
    a = [_c(x) for x in (psi, pi, phi, lapse, shift, gamma1, gamma2, normal, normal_vector, xyz,
                         d_psi, d_pi, d_phi, dt_psi, dt_pi, dt_phi)]
    n = a[0].shape[0]
    out = np.zeros((5, n))
    _check(lib().orc_csw_cpsr(n, *[_p(x) for x in a], _p(out)))
    return out


def shell(r_inner=1.9, r_outer=20.0, ref_ang=2, ref_rad=3, n=10, mass=1.0, gamma1=0.0,
          gamma2=0.0):
    """Six-wedge spherical shell, (ref_ang, ref_ang, ref_rad) per wedge."""
    return OrcShell(r_inner, r_outer, ref_ang, ref_rad, n, mass, gamma1, gamma2)


def shell_num_elements(s):
    return int(lib().orc_shell_num_elements(ctypes.byref(s)))


def shell_geometry(s):
    """(xyz [E,3,N^3], inv_jac [E,9,N^3]) with inv_jac[3a+i] = d xi^a / d x^i."""
    E, np3 = shell_num_elements(s), s.n ** 3
    xyz = np.zeros((E, 3, np3))
    ij = np.zeros((E, 9, np3))
    _check(lib().orc_shell_geometry(ctypes.byref(s), _p(xyz), _p(ij)))
    return xyz, ij


def shell_connectivity(s):
    E = shell_num_elements(s)
    nbr = np.zeros((E, 6), dtype=np.int32)
    perm = np.zeros((E, 6, s.n * s.n), dtype=np.int32)
    ids = np.zeros(E, dtype=np.uint64)
    _check(lib().orc_shell_connectivity(ctypes.byref(s), _p(nbr), _p(perm), _p(ids)))
    return nbr, perm, ids


def shell_initial_data(s, r0=8.0, width=1.5):
    u = np.zeros((shell_num_elements(s), 5, s.n ** 3))
    _check(lib().orc_shell_initial_data(ctypes.byref(s), r0, width, _p(u)))
    return u


def shell_rhs(s, u, threads=0, fast=False):
    """Returns (dudt, excision_ok)."""
    u = _c(u)
    du = np.zeros_like(u)
    rc = lib(fast).orc_shell_rhs(ctypes.byref(s), _p(u), _p(du), threads)
    if rc < 0:
        _check(rc)
    return du, rc == 0


def shell_evolve(s, u, dt, steps, threads=0):
    u = _c(u).copy()
    rc = lib().orc_shell_evolve(ctypes.byref(s), dt, steps, _p(u), threads)
    if rc < 0:
        _check(rc)
    return u, rc == 0


def exponential_filter(n, alpha, half_power):
    F = np.zeros((n, n))
    _check(lib().orc_exponential_filter(n, alpha, half_power, _p(F)))
    return F


def filter_elements(elem_n, u, alpha, half_power):
    """Filtered copy of a state whose elements have extents elem_n."""
    en = np.ascontiguousarray(elem_n, dtype=np.int32)
    out = _c(u).copy()
    _check(lib().orc_filter_elements(len(en), _p(en), alpha, half_power, _p(out)))
    return out


NORM_NAMES = ("Max", "Min", "L2Norm", "L2IntegralNorm", "VolumeIntegral")


def observe_norms(bricks, points, u, subtract=None):
    """27 values: [5 * var + norm] for NORM_NAMES, then points, volume."""
    en = elem_points(bricks, points)
    arr = _bricks(bricks)
    out = np.zeros(27)
    u = _c(u)
    sub = None if subtract is None else _c(subtract)
    _check(lib().orc_observe_norms(len(bricks), ctypes.addressof(arr), _p(en), _p(u), _p(sub),
                                   _p(out)))
    return out


def shell_observe_norms(s, u):
    out = np.zeros(27)
    _check(lib().orc_shell_observe_norms(ctypes.byref(s), _p(_c(u)), _p(out)))
    return out


def lg(n):
    """Legendre-Gauss nodes and weights."""
    x, w = np.zeros(n), np.zeros(n)
    _check(lib().orc_lg(n, _p(x), _p(w)))
    return x, w


def lg_diff_matrix(n):
    D = np.zeros((n, n))
    _check(lib().orc_lg_diff_matrix(n, _p(D)))
    return D


def lg_boundary(n):
    """(interp to -1, interp to +1, lifting term -1, lifting term +1)."""
    a = [np.zeros(n) for _ in range(4)]
    _check(lib().orc_lg_boundary(n, *[_p(x) for x in a]))
    return tuple(a)


def coords_gauss(bricks, n):
    E = num_elements(bricks)
    xyz = np.zeros((E, 3, n ** 3))
    arr = _bricks(bricks)
    _check(lib().orc_coords_gauss(len(bricks), ctypes.addressof(arr), n, _p(xyz)))
    return xyz


def plane_wave_gauss(bricks, n, k, t=0.0):
    """PlaneWave initial data on the Gauss nodes, [E, 5, n^3]."""
    xyz = coords_gauss(bricks, n)
    k = np.asarray(k, dtype=np.float64)
    om = float(np.sqrt((k * k).sum()))
    ph = np.einsum("i,eip->ep", k, xyz) - om * t
    u = np.zeros((xyz.shape[0], 5, n ** 3))
    u[:, 0] = np.sin(ph)
    u[:, 1] = om * np.cos(ph)
    for d in range(3):
        u[:, 2 + d] = k[d] * np.cos(ph)
    return u


def rhs_gauss(bricks, n, u, gamma2=0.0, threads=0):
    u = _c(u)
    out = np.zeros_like(u)
    arr = _bricks(bricks)
    _check(lib().orc_rhs_gauss(len(bricks), ctypes.addressof(arr), n, gamma2, _p(u), _p(out),
                               threads))
    return out


def evolve_gauss(bricks, n, u, dt, steps, gamma2=0.0, threads=0):
    u = _c(u).copy()
    arr = _bricks(bricks)
    _check(lib().orc_evolve_gauss(len(bricks), ctypes.addressof(arr), n, gamma2, dt, steps,
                                  _p(u), threads))
    return u


class refined:
    """A periodic block lattice with one refinement level per block (kept
    alive with its level array for the ctypes calls)."""

    def __init__(self, blocks, levels, lo=(0.0, 0.0, 0.0), hi=(2 * math.pi,) * 3):
        self.levels = np.ascontiguousarray(levels, dtype=np.int32).ravel()
        self.s = OrcRefinedBrick()
        self.s.lo[:] = [float(v) for v in lo]
        self.s.hi[:] = [float(v) for v in hi]
        self.s.blocks[:] = [int(v) for v in blocks]
        self.s.level = self.levels.ctypes.data

    def num_elements(self):
        return int(lib().orc_refined_num_elements(ctypes.byref(self.s)))

    def index_maps(self):
        E = self.num_elements()
        ids = np.zeros(E, dtype=np.uint64)
        nbr = np.zeros((E, 6, 4), dtype=np.int32)
        ms = np.zeros((E, 6, 4, 2), dtype=np.int32)
        rc = lib().orc_refined_index_maps(ctypes.byref(self.s), _p(ids), _p(nbr), _p(ms))
        _check(rc)
        return ids, nbr, ms

    def coords(self, n):
        xyz = np.zeros((self.num_elements(), 3, n ** 3))
        _check(lib().orc_refined_coords(ctypes.byref(self.s), n, _p(xyz)))
        return xyz

    def plane_wave(self, n, k, t=0.0):
        xyz = self.coords(n)
        k = np.asarray(k, dtype=np.float64)
        om = float(np.sqrt((k * k).sum()))
        ph = np.einsum("i,eip->ep", k, xyz) - om * t
        u = np.zeros((xyz.shape[0], 5, n ** 3))
        u[:, 0] = np.sin(ph)
        u[:, 1] = om * np.cos(ph)
        for d in range(3):
            u[:, 2 + d] = k[d] * np.cos(ph)
        return u

    def rhs(self, n, u, gamma2=0.0, threads=0):
        u = _c(u)
        out = np.zeros_like(u)
        _check(lib().orc_refined_rhs(ctypes.byref(self.s), n, gamma2, _p(u), _p(out), threads))
        return out

    def evolve(self, n, u, dt, steps, gamma2=0.0, threads=0):
        u = _c(u).copy()
        _check(lib().orc_refined_evolve(ctypes.byref(self.s), n, gamma2, dt, steps, _p(u),
                                        threads))
        return u


def proj_half(n, upper):
    P, R = np.zeros((n, n)), np.zeros((n, n))
    _check(lib().orc_proj_half(n, int(upper), _p(P), _p(R)))
    return P, R


def amr_matrix(src, dst, child):
    """The dst x src 1D matrix of ProjectVariables: child 0 (p-projection),
    1 (LowerHalf) or 2 (UpperHalf)."""
    M = np.zeros((dst, src))
    _check(lib().orc_amr_matrix(int(src), int(dst), int(child), _p(M)))
    return M


def amr_project(n_vars, src, src_ext, dst_ext, child, u_in, in_off):
    """Target blocks from source blocks (ProjectVariables); returns the
    concatenated targets and their offsets."""
    src = np.ascontiguousarray(src, dtype=np.int32)
    src_ext = np.ascontiguousarray(src_ext, dtype=np.int32).reshape(-1, 3)
    dst_ext = np.ascontiguousarray(dst_ext, dtype=np.int32).reshape(-1, 3)
    child = np.ascontiguousarray(child, dtype=np.int8).reshape(-1, 3)
    sizes = n_vars * np.prod(dst_ext.astype(np.int64), axis=1)
    out_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    out = np.zeros(int(sizes.sum()))
    _check(lib().orc_amr_project(int(n_vars), len(src), _p(src), _p(src_ext), _p(dst_ext),
                                 _p(child), _p(_c(u_in)), _p(np.ascontiguousarray(in_off, dtype=np.int64)),
                                 _p(out), _p(out_off)))
    return out, out_off


# ---------------- Adams-Bashforth and local time stepping ----------------

def variable_coefficients(control_times, step_start, step_end):
    ct = np.ascontiguousarray(control_times, dtype=np.float64)
    out = np.zeros(len(ct))
    _check(lib().orc_variable_coefficients(len(ct), _p(ct), step_start, step_end, _p(out)))
    return out


def adams_coefficients(control_ticks, step_start, step_end, slab=1.0, ticks_per_slab=1):
    t = np.ascontiguousarray(control_ticks, dtype=np.int64)
    out = np.zeros(len(t))
    _check(lib().orc_adams_coefficients(len(t), _p(t), step_start, step_end, slab,
                                        ticks_per_slab, _p(out)))
    return out


def lts_coefficients(local_ids, remote_ids, step_start, step_end, order, slab=1.0,
                     ticks_per_slab=1):
    """local_ids / remote_ids: lists of (slab number, tick); order an int or
    (local, remote, small step) orders.  Returns a dict
    {(local id, remote id): coefficient}."""
    lo, ro, so = (order,) * 3 if np.ndim(order) == 0 else order
    ls = np.array([i[0] for i in local_ids], dtype=np.int64)
    lt = np.array([i[1] for i in local_ids], dtype=np.int64)
    rs = np.array([i[0] for i in remote_ids], dtype=np.int64)
    rt = np.array([i[1] for i in remote_ids], dtype=np.int64)
    m = 256
    ol = np.zeros(m, dtype=np.int32)
    orr = np.zeros(m, dtype=np.int32)
    oc = np.zeros(m)
    cnt = lib().orc_lts_coefficients(len(ls), _p(ls), _p(lt), len(rs), _p(rs), _p(rt),
                                      step_start, step_end, slab, ticks_per_slab, lo, ro, so, m,
                                      _p(ol), _p(orr), _p(oc))
    _check(min(cnt, 0))
    return {(tuple(local_ids[ol[i]]), tuple(remote_ids[orr[i]])): oc[i] for i in range(cnt)}


def evolve_adams(bricks, n, u, slab, n_slabs, order, levels=None, gamma2=0.0, threads=0):
    u = np.array(u, dtype=np.float64, copy=True)
    arr = _bricks(bricks)
    lv = None if levels is None else np.ascontiguousarray(levels, dtype=np.int32)
    _check(lib().orc_evolve_adams(len(bricks), ctypes.addressof(arr), n, gamma2, order, _p(lv),
                                  slab, n_slabs, _p(u), threads))
    return u


def evolve_adams_extents(bricks, elem_n, u, slab, n_slabs, order, levels=None, gamma2=0.0,
                         threads=0):
    """AdamsBashforth(order) with local time stepping on bricks whose
    elements have their own extents (p-nonconforming mortars)."""
    u = np.array(u, dtype=np.float64, copy=True)
    arr = _bricks(bricks)
    en = np.ascontiguousarray(elem_n, dtype=np.int32)
    lv = None if levels is None else np.ascontiguousarray(levels, dtype=np.int32)
    _check(lib().orc_evolve_adams_extents(len(bricks), ctypes.addressof(arr), _p(en), gamma2,
                                          order, _p(lv), slab, n_slabs, _p(u), threads))
    return u


def shell_evolve_adams(s, u, slab, n_slabs, order, levels=None, threads=0, filter=None):
    """AdamsBashforth(order) with local time stepping on the shell; filter =
    (alpha, half_power) applies the exponential filter to each element after
    every one of its steps."""
    u = np.array(u, dtype=np.float64, copy=True)
    lv = None if levels is None else np.ascontiguousarray(levels, dtype=np.int32)
    if filter is None:
        _check(lib().orc_shell_evolve_adams(ctypes.addressof(s), order, _p(lv), slab, n_slabs,
                                            _p(u), threads))
    else:
        _check(lib().orc_shell_evolve_adams_filtered(ctypes.addressof(s), order, _p(lv), slab,
                                                     n_slabs, float(filter[0]), int(filter[1]),
                                                     _p(u), threads))
    return u


# ---------------- time bookkeeping (pure Python, exact fractions) ----------------

class TimeStepIdOracle:
    """TimeStepId restated with exact fractions (test infrastructure).

    Time: a slab [start, end] and a fraction f of it, value (1 - f) start +
    f end with each fraction converted to double (Time.cpp:96-98,
    Rational.cpp:41-43).  next_step / next_substep / canonicalize follow
    TimeStepId.cpp:65-97; Slab::advance / retreat follow Slab.cpp:31-33."""

    def __init__(self, forward, slab_number, slab_start, slab_end, frac):
        from fractions import Fraction
        self.slab_number = slab_number
        self.slab = (slab_start, slab_end)
        self.frac = Fraction(frac)
        self.substep = 0
        self.size = Fraction(1 if forward else -1)
        self.substep_time = self._value(self.frac)
        self._canonicalize()

    def _value(self, f):
        start, end = self.slab
        return float(1 - f) * start + float(f) * end

    def _canonicalize(self):
        forward = self.size > 0
        if (self.frac == 1) if forward else (self.frac == 0):
            assert self.substep == 0
            start, end = self.slab
            if forward:
                self.slab = (end, end + (end - start))
                self.frac = self.frac - 1
            else:
                self.slab = (start - (end - start), start)
                self.frac = self.frac + 1
            self.slab_number += 1

    def _copy(self):
        import copy
        return copy.copy(self)

    def next_step(self, size):
        from fractions import Fraction
        out = self._copy()
        out.frac = self.frac + Fraction(size)
        assert 0 <= out.frac <= 1
        out.substep = 0
        out.size = Fraction(1 if size > 0 else -1)
        out.substep_time = out._value(out.frac)
        out._canonicalize()
        return out

    def next_substep(self, size, step_fraction):
        from fractions import Fraction
        end = self.frac + Fraction(size)
        assert 0 <= end <= 1
        out = self._copy()
        out.substep = self.substep + 1
        out.size = Fraction(size)
        out.substep_time = ((1.0 - step_fraction) * self._value(self.frac)
                            + step_fraction * self._value(end))
        return out

    def key(self):
        size = self.size
        return (self.slab_number, self.slab[0], self.slab[1], self.frac.numerator,
                self.frac.denominator, self.substep, size.numerator, size.denominator,
                self.substep_time)


def rk3_next_time_id(current, size):
    """Rk3HesthavenSsp::next_time_id, Rk3HesthavenSsp.cpp:36-48."""
    if current.substep == 0:
        return current.next_substep(size, 1.0)
    if current.substep == 1:
        return current.next_substep(size, 0.5)
    if current.substep == 2:
        return current.next_step(size)
    raise ValueError("Bad id")
