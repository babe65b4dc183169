"""Python mirror of SpECTRE's DG scalar-wave operator surface over libdgsw.so.

The classes keep the reference's names and argument meaning:

  ScalarWaveSystem   ScalarWave::System<3>            (Evolution/Systems/ScalarWave/System.hpp:39-57)
  TimeDerivative     ScalarWave::TimeDerivative<3>    (Evolution/Systems/ScalarWave/TimeDerivative.cpp:13-45)
  UpwindPenalty      ScalarWave::BoundaryCorrections::UpwindPenalty<3>
                                                      (.../BoundaryCorrections/UpwindPenalty.cpp:35-205)
  Rk3HesthavenSsp    TimeSteppers::Rk3HesthavenSsp    (Time/TimeSteppers/Rk3HesthavenSsp.cpp:21-81)
  DgEvolution        the per-element DG step of EvolveScalarWave (ComputeTimeDerivative +
                     ApplyBoundaryCorrections + UpdateU) for every element of one or more
                     periodic bricks, owned by one libdgsw handle on one GPU.

Every call goes through the C ABI in include/dgsw.h.  There is no CPU
fallback: if the library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdgsw.so")

DGSW_OK = 0
STATUS_NAMES = {
    -1: "DGSW_ERR_ARGUMENT",
    -2: "DGSW_ERR_CUDA",
    -3: "DGSW_ERR_UNSUPPORTED",
    -4: "DGSW_ERR_NOT_FINITE",
    -5: "DGSW_ERR_NO_DEVICE",
    -6: "DGSW_ERR_DEVICE_TIMEOUT",
    -7: "DGSW_ERR_CFL",
}
PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_DOUBLE_FLOAT = 2  # FP64 state, double-float (hi + lo FP32) arithmetic
N_VARS = 5  # Psi, Pi, Phi_x, Phi_y, Phi_z
N_PACKAGED = 16  # UpwindPenalty dg_package_field_tags doubles per face point
STAGE_VARIANTS = 4  # DGSW_STAGE_VARIANTS: launch configurations of the FP64 stage


class DgswError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, message))
        self.status = status


class DgswBrick(ctypes.Structure):
    _fields_ = [("lower", ctypes.c_double * 3), ("upper", ctypes.c_double * 3),
                ("elements", ctypes.c_int32 * 3)]


class DgswRefinedBrick(ctypes.Structure):
    _fields_ = [("lower", ctypes.c_double * 3), ("upper", ctypes.c_double * 3),
                ("blocks", ctypes.c_int32 * 3), ("levels", ctypes.POINTER(ctypes.c_int32))]


class DgswShell(ctypes.Structure):
    _fields_ = [("inner_radius", ctypes.c_double), ("outer_radius", ctypes.c_double),
                ("refinement_angular", ctypes.c_int32), ("refinement_radial", ctypes.c_int32),
                ("radial_distribution", ctypes.c_int32), ("mass", ctypes.c_double),
                ("gamma1", ctypes.c_double)]


class DgswConfig(ctypes.Structure):
    _fields_ = [("system", ctypes.c_int32), ("boundary_correction", ctypes.c_int32),
                ("time_stepper", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("n_instances", ctypes.c_int32), ("bricks", ctypes.POINTER(DgswBrick)),
                ("points_per_element", ctypes.POINTER(ctypes.c_int32)),
                ("uniform_points", ctypes.c_int32), ("gamma2", ctypes.c_double),
                ("device", ctypes.c_int32), ("shell", ctypes.POINTER(DgswShell)),
                ("quadrature", ctypes.c_int32),
                ("refined", ctypes.POINTER(DgswRefinedBrick)),
                ("stepper_order", ctypes.c_int32),
                ("step_levels", ctypes.POINTER(ctypes.c_int32))]


class DgswTimeStepId(ctypes.Structure):
    _fields_ = [("slab_number", ctypes.c_int64), ("slab_start", ctypes.c_double),
                ("slab_end", ctypes.c_double), ("step_num", ctypes.c_int32),
                ("step_den", ctypes.c_int32), ("substep", ctypes.c_int32),
                ("size_num", ctypes.c_int32), ("size_den", ctypes.c_int32),
                ("substep_time", ctypes.c_double)]

    def key(self):
        return (self.slab_number, self.slab_start, self.slab_end, self.step_num,
                self.step_den, self.substep, self.size_num, self.size_den, self.substep_time)


class DgswAdamsJob(ctypes.Structure):
    _fields_ = [("launch", ctypes.c_int32), ("level", ctypes.c_int32),
                ("update", ctypes.c_int32), ("reset", ctypes.c_int32),
                ("rec_slot", ctypes.c_int32), ("n_vol", ctypes.c_int32),
                ("vol_slot", ctypes.c_int32 * 8), ("vol_c", ctypes.c_double * 8),
                ("n_loc", ctypes.c_int32 * 4), ("loc_slot", (ctypes.c_int32 * 8) * 4),
                ("loc_c", (ctypes.c_double * 8) * 4), ("n_rem", ctypes.c_int32 * 4),
                ("rem_slot", (ctypes.c_int32 * 16) * 4), ("rem_c", (ctypes.c_double * 16) * 4)]


SYSTEM_SCALAR_WAVE = 0
SYSTEM_CURVED_SCALAR_WAVE = 1
RADIAL_DISTRIBUTIONS = {"linear": 0, "logarithmic": 1}
QUADRATURES = {"gauss_lobatto": 0, "gauss": 1}
TIME_STEPPERS = {"rk3_hesthaven_ssp": 0, "adams_bashforth": 1}


_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_SIGNATURES = {
    "dgsw_abi_version": (_I, []),
    "dgsw_last_error": (ctypes.c_char_p, [_P]),
    "dgsw_create": (_I, [ctypes.POINTER(DgswConfig), ctypes.POINTER(_P)]),
    "dgsw_destroy": (_I, [_P]),
    "dgsw_sizes": (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "dgsw_stream": (_P, [_P]),
    "dgsw_synchronize": (_I, [_P]),
    "dgsw_set_state": (_I, [_P, _P]),
    "dgsw_get_state": (_I, [_P, _P]),
    "dgsw_set_state_device": (_I, [_P, _P]),
    "dgsw_get_state_device": (_I, [_P, _P]),
    "dgsw_set_initial_data": (_I, [_P, _I, _P, _D]),
    "dgsw_rhs": (_I, [_P, _P, _P]),
    "dgsw_rhs_device": (_I, [_P, _P, _P]),
    "dgsw_volume_rhs_device": (_I, [_P, _P, _P]),
    "dgsw_package_data_device": (_I, [_I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "dgsw_boundary_terms_device": (_I, [_I64, _P, _P, _P, _P]),
    "dgsw_step": (_I, [_P, _I, _D]),
    "dgsw_step_host": (_I, [_P, _P, _I, _D]),
    "dgsw_set_exponential_filter": (_I, [_P, _D, _I, _I]),
    "dgsw_observe_norms": (_I, [_P, _P, _P, _P]),
    "dgsw_check_device_timeout": (_I, [_P, _D]),
    "dgsw_autotune": (_I, [_P, _I, ctypes.POINTER(_I), _P]),
    "dgsw_tune": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), _P]),
    "dgsw_observe_plane_wave_errors": (_I, [_P, _P, _D, _P]),
    "dgsw_exponential_filter_matrix": (_I, [_I, _D, _I, _P]),
    "dgsw_substep": (_I, [_P, _I, _D]),
    "dgsw_lgl_points_weights": (_I, [_I, _P, _P]),
    "dgsw_differentiation_matrix": (_I, [_I, _P]),
    "dgsw_mortar_projections": (_I, [_I, _I, _P, _P]),
    "dgsw_index_maps": (_I, [ctypes.POINTER(DgswConfig), _P, _P, _P]),
    "dgsw_count_elements": (_I, [ctypes.POINTER(DgswConfig), ctypes.POINTER(_I64),
                                 ctypes.POINTER(_I64)]),
    "dgsw_shell_geometry": (_I, [ctypes.POINTER(DgswConfig), _P, _P, _P]),
    "dgsw_gauss_spectral": (_I, [_I, _P, _P, _P, _P, _P, _P, _P]),
    "dgsw_refined_mortars": (_I, [ctypes.POINTER(DgswConfig), _P, _P]),
    "dgsw_half_projections": (_I, [_I, _I, _P, _P]),
    "dgsw_amr_matrix": (_I, [_I, _I, _I, _P]),
    "dgsw_amr_project_device": (_I, [_P, _I, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "dgsw_adjoint_rhs_device": (_I, [_P, _P, _P]),
    "dgsw_set_samples": (_I, [_P, _I, _P]),
    "dgsw_sample_psi": (_I, [_P, _P]),
    "dgsw_misfit_forward": (_I, [_P, _I, _I, _D, _P, ctypes.POINTER(_D)]),
    "dgsw_misfit_adjoint": (_I, [_P, _P]),
    "dgsw_adjoint_autotune": (_I, [_P, _I, ctypes.POINTER(_I), _P]),
    "dgsw_step_noalloc": (_I, [ctypes.POINTER(DgswBrick), _I, _D, _P, _I, _D, _P]),
    "dgsw_adams_info": (_I, [_P, _P, _P, _P, _P]),
    "dgsw_cfl_steps": (_I, [ctypes.POINTER(DgswConfig), _D, _P, _P]),
    "dgsw_set_guards": (_I, [_P, _D, _I]),
    "dgsw_check_finite": (_I, [_P, ctypes.POINTER(_I64)]),
    "dgsw_adams_coefficients": (_I, [_I, _P, _I64, _I64, _D, _I64, _P]),
    "dgsw_lts_coefficients": (_I, [_I, _P, _P, _I, _P, _P, _I64, _I64, _D, _I64, _I, _I, _I,
                                   _I, _P, _P, _P]),
    "dgsw_adams_schedule": (_I, [_I, _P, _P, _D, _I, _I, _P, _P, _P, _P]),
    "dgsw_time_step_id": (_I, [_I, _I64, _D, _D, ctypes.c_int32, ctypes.c_int32,
                               ctypes.POINTER(DgswTimeStepId)]),
    "dgsw_next_time_id": (_I, [_I, ctypes.POINTER(DgswTimeStepId), ctypes.c_int32,
                               ctypes.c_int32, ctypes.POINTER(DgswTimeStepId)]),
    "dgsw_substep_time_fraction": (_I, [_I, _I, ctypes.POINTER(_D)]),
    "dgsw_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "dgsw_noalloc_last_error": (ctypes.c_char_p, []),
}

_lib_handle = None


def lib() -> ctypes.CDLL:
    """The loaded libdgsw.so.  Raises if it has not been built."""
    global _lib_handle
    if _lib_handle is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libdgsw.so is not built (%s); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib_handle = L
    return _lib_handle


def exported_symbols() -> Sequence[str]:
    return tuple(_SIGNATURES)


def _check(status: int, handle=None):
    if status != DGSW_OK:
        msg = lib().dgsw_last_error(handle)
        raise DgswError(status, msg.decode() if msg else "")


def _torch_ready(*tensors):
    """Orders work queued by torch on its current stream before a library call
    that reads or writes these device tensors on the handle's own stream."""
    for t in tensors:
        if t is not None and hasattr(t, "is_cuda") and t.is_cuda:
            import torch
            torch.cuda.current_stream(t.device).synchronize()
            return


def _ptr(a) -> int:
    """Address of a numpy array or torch tensor (contiguous)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous()
        return a.data_ptr()
    raise TypeError("expected numpy array or torch tensor")


# ----------------------------------------------------------------- spectral


def lgl_points_weights(n: int):
    """Spectral::collocation_points / quadrature_weights <Legendre, GaussLobatto>."""
    x = np.zeros(n)
    w = np.zeros(n)
    _check(lib().dgsw_lgl_points_weights(n, _ptr(x), _ptr(w)))
    return x, w


def differentiation_matrix(n: int) -> np.ndarray:
    """Spectral::differentiation_matrix (row-major n x n)."""
    D = np.zeros((n, n))
    _check(lib().dgsw_differentiation_matrix(n, _ptr(D)))
    return D


def exponential_filter_matrix(n: int, alpha: float, half_power: int) -> np.ndarray:
    """Spectral::filtering::exponential_filter on n LGL points (row-major)."""
    F = np.zeros((n, n))
    _check(lib().dgsw_exponential_filter_matrix(n, float(alpha), int(half_power), _ptr(F)))
    return F


def gauss_spectral(n: int):
    """Legendre-Gauss tables: dict of x, w, D, interp_lower, interp_upper,
    lift_lower, lift_upper (Spectral::Quadrature::Gauss)."""
    out = {k: np.zeros(n) for k in ("x", "w", "interp_lower", "interp_upper", "lift_lower",
                                     "lift_upper")}
    out["D"] = np.zeros((n, n))
    _check(lib().dgsw_gauss_spectral(n, _ptr(out["x"]), _ptr(out["w"]), _ptr(out["D"]),
                                     _ptr(out["interp_lower"]), _ptr(out["interp_upper"]),
                                     _ptr(out["lift_lower"]), _ptr(out["lift_upper"])))
    return out


def mortar_projections(n_face: int, n_mortar: int):
    """(face->mortar [nm x ne], mortar->face [ne x nm]) for ChildSize::Full."""
    a = np.zeros((n_mortar, n_face))
    b = np.zeros((n_face, n_mortar))
    _check(lib().dgsw_mortar_projections(n_face, n_mortar, _ptr(a), _ptr(b)))
    return a, b


# ------------------------------------------------------------------ domain


@dataclass
class Brick:
    """Periodic [lower, upper]^3 split into elements[d] elements along d."""
    elements: Sequence[int]
    lower: Sequence[float] = (0.0, 0.0, 0.0)
    upper: Sequence[float] = (2 * math.pi, 2 * math.pi, 2 * math.pi)


@dataclass
class RefinedBrick:
    """Periodic lattice of blocks on [lower, upper]^3 (blocks x fastest); block
    k has 2^levels[k] elements per axis; face-sharing blocks differ by at most
    one level (h-nonconforming 2:1 mortars)."""
    blocks: Sequence[int]
    levels: Sequence[int]
    lower: Sequence[float] = (0.0, 0.0, 0.0)
    upper: Sequence[float] = (2 * math.pi, 2 * math.pi, 2 * math.pi)


@dataclass
class Shell:
    """Spherical shell of six cubed-sphere wedges (Domain::Creators::Sphere
    without its interior) on a Schwarzschild background in Kerr-Schild
    coordinates; each wedge has 2^refinement_angular x 2^refinement_angular x
    2^refinement_radial elements."""
    inner_radius: float = 1.9
    outer_radius: float = 20.0
    refinement_angular: int = 2
    refinement_radial: int = 3
    radial_distribution: str = "logarithmic"
    mass: float = 1.0
    gamma1: float = 0.0


class _ConfigHolder:
    """Keeps the ctypes arrays a DgswConfig points to alive."""

    def __init__(self, bricks, points, precision=PRECISION_FP64, gamma2=0.0, device=0,
                 quadrature="gauss_lobatto", time_stepper="rk3_hesthaven_ssp", order=0,
                 step_levels=None):
        self.shell = None
        self.refined = None
        if isinstance(bricks, RefinedBrick):
            rb = bricks
            self.levels = np.ascontiguousarray(rb.levels, dtype=np.int32).ravel()
            self.refined = DgswRefinedBrick()
            self.refined.lower[:] = [float(v) for v in rb.lower]
            self.refined.upper[:] = [float(v) for v in rb.upper]
            self.refined.blocks[:] = [int(v) for v in rb.blocks]
            self.refined.levels = self.levels.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            bricks = []
        if isinstance(bricks, Shell):
            sh = bricks
            self.shell = DgswShell(float(sh.inner_radius), float(sh.outer_radius),
                                   int(sh.refinement_angular), int(sh.refinement_radial),
                                   RADIAL_DISTRIBUTIONS[sh.radial_distribution],
                                   float(sh.mass), float(sh.gamma1))
            bricks = []
        self.bricks = (DgswBrick * max(1, len(bricks)))()
        for i, b in enumerate(bricks):
            self.bricks[i].lower[:] = [float(v) for v in b.lower]
            self.bricks[i].upper[:] = [float(v) for v in b.upper]
            self.bricks[i].elements[:] = [int(v) for v in b.elements]
        self.points = None
        uniform = 0
        if np.ndim(points) == 0:
            uniform = int(points)
        else:
            self.points = np.ascontiguousarray(points, dtype=np.int32)
        self.cfg = DgswConfig()
        self.cfg.system = SYSTEM_CURVED_SCALAR_WAVE if self.shell else SYSTEM_SCALAR_WAVE
        self.cfg.boundary_correction = 0
        self.cfg.time_stepper = 0
        self.cfg.precision = precision
        self.cfg.n_instances = 1 if (self.shell or self.refined) else len(bricks)
        self.cfg.bricks = ctypes.cast(self.bricks, ctypes.POINTER(DgswBrick))
        self.cfg.points_per_element = (
            self.points.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            if self.points is not None else None)
        self.cfg.uniform_points = uniform
        self.cfg.gamma2 = float(gamma2)
        self.cfg.device = device
        self.cfg.shell = ctypes.pointer(self.shell) if self.shell else None
        self.cfg.quadrature = QUADRATURES[quadrature]
        self.cfg.refined = ctypes.pointer(self.refined) if self.refined else None
        self.cfg.time_stepper = TIME_STEPPERS[time_stepper]
        self.cfg.stepper_order = int(order)
        self.step_levels = None
        if step_levels is not None:
            self.step_levels = np.ascontiguousarray(step_levels, dtype=np.int32).ravel()
        self.cfg.step_levels = (
            self.step_levels.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            if self.step_levels is not None else None)


def refined_mortars(refined: "RefinedBrick", points: int):
    """(neighbour slots [E, 6, 4], mortar sizes [E, 6, 4, 2]: 0 Full,
    1 LowerHalf, 2 UpperHalf) of a refined lattice."""
    h = _ConfigHolder(refined, points)
    ne, nd = _I64(), _I64()
    _check(lib().dgsw_count_elements(ctypes.byref(h.cfg), ctypes.byref(ne), ctypes.byref(nd)))
    E = ne.value
    slots = np.zeros((E, 6, 4), dtype=np.int32)
    sizes = np.zeros((E, 6, 4, 2), dtype=np.int32)
    _check(lib().dgsw_refined_mortars(ctypes.byref(h.cfg), _ptr(slots), _ptr(sizes)))
    return slots, sizes


def half_projections(n: int, upper: bool):
    """(parent -> child interpolation, child -> parent restriction), n x n."""
    P, R = np.zeros((n, n)), np.zeros((n, n))
    _check(lib().dgsw_half_projections(n, int(upper), _ptr(P), _ptr(R)))
    return P, R


AMR_FULL, AMR_LOWER_HALF, AMR_UPPER_HALF = 0, 1, 2


def amr_matrix(src_extent: int, dst_extent: int, child: int = AMR_FULL):
    """The dst x src 1D matrix of amr::projectors::ProjectVariables along one
    dimension (host only): AMR_FULL p-projection, AMR_LOWER_HALF /
    AMR_UPPER_HALF h-refinement into that half."""
    M = np.zeros((int(dst_extent), int(src_extent)))
    _check(lib().dgsw_amr_matrix(int(src_extent), int(dst_extent), int(child), _ptr(M)))
    return M


def amr_project(owner, n_vars, u_in, in_offset, src, src_extents, dst_extents, child):
    """ProjectVariables on the device through dgsw_amr_project_device.

    owner: any open DgEvolution (its device and stream are used).  u_in: a
    CUDA tensor of float64 holding the source blocks at in_offset (doubles).
    src: source block of each target; src_extents / dst_extents / child:
    3 per target.  Returns (CUDA float64 tensor of the targets, concatenated
    in order, and their offsets)."""
    import torch
    src = np.ascontiguousarray(src, dtype=np.int32)
    se = np.ascontiguousarray(src_extents, dtype=np.int32).reshape(-1, 3)
    de = np.ascontiguousarray(dst_extents, dtype=np.int32).reshape(-1, 3)
    ch = np.ascontiguousarray(child, dtype=np.int8).reshape(-1, 3)
    ino = np.ascontiguousarray(in_offset, dtype=np.int64)
    if not (len(src) == len(se) == len(de) == len(ch)):
        raise ValueError("one source index and three extents / child sizes per target")
    sizes = int(n_vars) * np.prod(de.astype(np.int64), axis=1)
    out_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    assert u_in.is_cuda and u_in.dtype == torch.float64 and u_in.is_contiguous()
    out = torch.empty(int(sizes.sum()), dtype=torch.float64, device=u_in.device)
    _check(lib().dgsw_amr_project_device(owner.handle, int(n_vars), len(ino), _ptr(ino),
                                          u_in.data_ptr(), len(src), _ptr(src), _ptr(se),
                                          _ptr(de), _ptr(ch), _ptr(out_off), out.data_ptr()),
           owner.handle)
    return out, out_off


def cfl_steps(bricks, points, safety_factor=1.0, time_stepper="rk3_hesthaven_ssp", order=3,
              quadrature="gauss_lobatto", gamma2=0.0):
    """StepChoosers::Cfl per element (host-only): returns the array of
    element steps.  bricks: Brick list, Shell or RefinedBrick."""
    if isinstance(bricks, Brick):
        bricks = [bricks]
    holder = _ConfigHolder(bricks, points, gamma2=gamma2, quadrature=quadrature,
                           time_stepper=time_stepper, order=order)
    ne, nd = _I64(), _I64()
    _check(lib().dgsw_count_elements(ctypes.byref(holder.cfg), ctypes.byref(ne), ctypes.byref(nd)))
    out = np.zeros(ne.value)
    m = ctypes.c_double()
    _check(lib().dgsw_cfl_steps(ctypes.byref(holder.cfg), float(safety_factor), _ptr(out),
                                ctypes.byref(m)))
    return out


def levels_from_cfl(element_steps, slab):
    """Step levels for AdamsBashforth local time stepping: the smallest l in
    0..3 with slab / 2^l within each element's Cfl step."""
    s = np.asarray(element_steps, dtype=np.float64)
    lv = np.ceil(np.log2(np.maximum(slab / s, 1.0))).astype(np.int32)
    if np.any(lv > 3):
        raise ValueError("the slab needs more than 3 levels below it")
    return lv


def adams_coefficients(control_ticks, step_start, step_end, slab=1.0, ticks_per_slab=1):
    """adams_coefficients::coefficients for control times given in ticks."""
    t = np.ascontiguousarray(control_ticks, dtype=np.int64)
    out = np.zeros(len(t))
    _check(lib().dgsw_adams_coefficients(len(t), _ptr(t), int(step_start), int(step_end),
                                         float(slab), int(ticks_per_slab), _ptr(out)))
    return out


def lts_coefficients(local_ids, remote_ids, step_start, step_end, order, slab=1.0,
                     ticks_per_slab=1):
    """adams_lts::lts_coefficients; ids are (slab number, tick) pairs, order
    an int or (local, remote, small step) orders.  Returns
    {(local id, remote id): coefficient}."""
    lo, ro, so = (order,) * 3 if np.ndim(order) == 0 else order
    ls = np.array([i[0] for i in local_ids], dtype=np.int64)
    lt = np.array([i[1] for i in local_ids], dtype=np.int64)
    rs = np.array([i[0] for i in remote_ids], dtype=np.int64)
    rt = np.array([i[1] for i in remote_ids], dtype=np.int64)
    m = 256
    ol, orr, oc = np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros(m)
    cnt = lib().dgsw_lts_coefficients(len(ls), _ptr(ls), _ptr(lt), len(rs), _ptr(rs), _ptr(rt),
                                      int(step_start), int(step_end), float(slab),
                                      int(ticks_per_slab), lo, ro, so, m, _ptr(ol), _ptr(orr),
                                      _ptr(oc))
    if cnt < 0:
        _check(cnt)
    return {(tuple(local_ids[ol[i]]), tuple(remote_ids[orr[i]])): oc[i] for i in range(cnt)}


def adams_schedule(order, level_counts, adjacency, slab, n_slabs, max_jobs=100000):
    """The device schedule of n_slabs slabs: (jobs, ticks per slab, ring
    slots); jobs is a list of DgswAdamsJob."""
    cnt = np.zeros(4, np.int64)
    cnt[:len(level_counts)] = level_counts
    adj = np.zeros((4, 4), np.int32)
    a = np.asarray(adjacency, dtype=np.int32)
    adj[:a.shape[0], :a.shape[1]] = a
    adj = np.ascontiguousarray(adj.ravel())
    jobs = (DgswAdamsJob * max_jobs)()
    nj, S, ring = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
    _check(lib().dgsw_adams_schedule(int(order), _ptr(cnt), _ptr(adj), float(slab), int(n_slabs),
                                     max_jobs, ctypes.addressof(jobs), ctypes.byref(nj),
                                     ctypes.byref(S), ctypes.byref(ring)))
    return list(jobs[:nj.value]), S.value, ring.value


def shell_geometry(shell: "Shell", points: int):
    """(xyz [E,3,N^3], inverse Jacobian [E,9,N^3] with component 3a+i =
    d xi^a / d x^i, face permutations [E,6,N^2]) of a shell (host, FP64)."""
    h = _ConfigHolder(shell, points)
    ne, nd = _I64(), _I64()
    _check(lib().dgsw_count_elements(ctypes.byref(h.cfg), ctypes.byref(ne), ctypes.byref(nd)))
    E, np3 = ne.value, points ** 3
    xyz = np.zeros((E, 3, np3))
    ij = np.zeros((E, 9, np3))
    perm = np.zeros((E, 6, points * points), dtype=np.int32)
    _check(lib().dgsw_shell_geometry(ctypes.byref(h.cfg), _ptr(xyz), _ptr(ij), _ptr(perm)))
    return xyz, ij, perm


def index_maps(bricks, points):
    """(element_ids uint64, neighbors int32 [E,6], mortar extents int32 [E,6], fits)."""
    h = _ConfigHolder(bricks, points)
    ne = _I64()
    nd = _I64()
    _check(lib().dgsw_count_elements(ctypes.byref(h.cfg), ctypes.byref(ne), ctypes.byref(nd)))
    E = ne.value
    ids = np.zeros(E, dtype=np.uint64)
    nbr = np.zeros((E, 6), dtype=np.int32)
    mort = np.zeros((E, 6), dtype=np.int32)
    st = lib().dgsw_index_maps(ctypes.byref(h.cfg), _ptr(ids), _ptr(nbr), _ptr(mort))
    if st not in (DGSW_OK, -3):
        _check(st)
    return ids, nbr, mort, st == DGSW_OK


# ------------------------------------------------------------------ system


class ScalarWaveSystem:
    """ScalarWave::System<3>: variables {Psi, Pi, Phi_i}, no fluxes."""
    volume_dim = 3
    variables = ("Psi", "Pi", "Phi")
    number_of_components = N_VARS
    has_primitive_and_conservative_vars = False


class CurvedScalarWaveSystem(ScalarWaveSystem):
    """CurvedScalarWave::System<3> (CurvedScalarWave/System.hpp:24-62): the
    same variables on a fixed background spacetime (lapse, shift, inverse
    spatial metric and their derivatives), constraint damping gamma1, gamma2."""
    spacetime_variables = ("Lapse", "Shift", "InverseSpatialMetric", "DerivLapse",
                           "DerivShift", "TraceSpatialChristoffel", "TraceExtrinsicCurvature")


class UpwindPenalty:
    """ScalarWave::BoundaryCorrections::UpwindPenalty<3> on device face data.

    Fields are torch CUDA float64 tensors: scalars of shape [npts], covectors
    of shape [3, npts].  Packaged data is a [16, npts] tensor in
    dg_package_field_tags order.
    """

    def dg_package_data(self, psi, pi, phi, constraint_gamma2, normal_covector,
                        mesh_velocity=None, normal_dot_mesh_velocity=None, stream=None):
        import torch
        npts = psi.numel()
        out = torch.empty((N_PACKAGED, npts), dtype=torch.float64, device=psi.device)
        if stream is None:
            _torch_ready(psi)
        _check(lib().dgsw_package_data_device(
            npts, _ptr(psi), _ptr(pi), _ptr(phi), _ptr(constraint_gamma2),
            _ptr(normal_covector),
            _ptr(normal_dot_mesh_velocity) if normal_dot_mesh_velocity is not None else None,
            _ptr(out), stream))
        # max over the char speeds, as the reference's return value
        max_speed = float(out[13:16].max()) if npts else float("-inf")
        return out, max_speed

    def dg_boundary_terms(self, packaged_int, packaged_ext, dg_formulation="StrongInertial",
                          stream=None):
        import torch
        npts = packaged_int.shape[1]
        out = torch.empty((N_VARS, npts), dtype=torch.float64, device=packaged_int.device)
        if stream is None:
            _torch_ready(packaged_int)
        _check(lib().dgsw_boundary_terms_device(npts, _ptr(packaged_int), _ptr(packaged_ext),
                                                _ptr(out), stream))
        return out


class Rk3HesthavenSsp:
    """TimeSteppers::Rk3HesthavenSsp: 3-stage, 3rd-order SSP Runge-Kutta."""

    def order(self) -> int:
        return 3

    def number_of_substeps(self) -> int:
        return 3

    def number_of_past_steps(self) -> int:
        return 0

    def stable_step(self) -> float:
        c = (4.0 + math.sqrt(17.0)) ** (1.0 / 3.0)
        return 0.5 * (1.0 + c - 1.0 / c)

    def substep_time_fractions(self):
        """Fractions of dt at which substeps 0, 1, 2 evaluate the RHS
        (dgsw_substep_time_fraction)."""
        out = []
        for k in range(self.number_of_substeps()):
            f = ctypes.c_double()
            _check(lib().dgsw_substep_time_fraction(TIME_STEPPERS["rk3_hesthaven_ssp"], k,
                                                    ctypes.byref(f)))
            out.append(f.value)
        return tuple(out)

    def next_time_id(self, current, step_num, step_den):
        """Rk3HesthavenSsp::next_time_id (Rk3HesthavenSsp.cpp:36-48) with a step
        of step_num/step_den of the slab."""
        return next_time_id("rk3_hesthaven_ssp", current, step_num, step_den)


def time_step_id(slab_number, slab_start, slab_end, num, den, time_runs_forward=True):
    """TimeStepId at the start of a step at fraction num/den of the slab."""
    out = DgswTimeStepId()
    _check(lib().dgsw_time_step_id(int(bool(time_runs_forward)), slab_number, slab_start,
                                   slab_end, num, den, ctypes.byref(out)))
    return out


def next_time_id(time_stepper, current, step_num, step_den):
    """TimeStepper::next_time_id of a DgswTimeStepId (dgsw_next_time_id)."""
    out = DgswTimeStepId()
    _check(lib().dgsw_next_time_id(TIME_STEPPERS[time_stepper], ctypes.byref(current),
                                   step_num, step_den, ctypes.byref(out)))
    return out


class DgEvolution:
    """All elements of one or more periodic bricks on one GPU (one handle), or
    of one spherical shell (pass a Shell: the CurvedScalarWave system)."""

    def __init__(self, bricks, points, precision=PRECISION_FP64, gamma2=0.0, device=0,
                 quadrature="gauss_lobatto", time_stepper="rk3_hesthaven_ssp", order=3,
                 step_levels=None):
        """time_stepper "adams_bashforth": AdamsBashforth of the given order
        with local time stepping; step_levels (one per element, 0..3, or
        None) make element e step slab / 2^step_levels[e], and step(dt)
        advances slabs of duration dt."""
        if isinstance(bricks, Brick):
            bricks = [bricks]
        self._cfg = _ConfigHolder(bricks, points, precision, gamma2, device, quadrature,
                                  time_stepper, order, step_levels)
        self.quadrature = quadrature
        self.time_stepper = time_stepper
        h = _P()
        _check(lib().dgsw_create(ctypes.byref(self._cfg.cfg), ctypes.byref(h)))
        self._h = h
        ne, nd, npt = _I64(), _I64(), _I64()
        _check(lib().dgsw_sizes(h, ctypes.byref(ne), ctypes.byref(nd), ctypes.byref(npt)), h)
        self.n_elements = ne.value
        self.state_size = nd.value
        self.grid_points = npt.value
        self.bricks = [] if isinstance(bricks, (Shell, RefinedBrick)) else list(bricks)
        self.points = points
        self.precision = precision
        self.gamma2 = gamma2
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            lib().dgsw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def stream_ptr(self) -> int:
        return lib().dgsw_stream(self._h) or 0

    def set_guards(self, cfl_safety_factor: float = 0.0, check_finite: bool = False):
        """dgsw_step refuses steps longer than the Cfl step (factor > 0) and
        reports NaN / Inf in the state afterwards (check_finite)."""
        _check(lib().dgsw_set_guards(self._h, float(cfl_safety_factor), int(bool(check_finite))),
               self._h)

    def first_non_finite_element(self) -> int:
        """The first element holding a NaN or Inf, -1 if none."""
        v = _I64()
        _check(lib().dgsw_check_finite(self._h, ctypes.byref(v)), self._h)
        return v.value

    def adams_info(self):
        """AdamsBashforth handles: dict of ring_slots, ticks_per_slab,
        rhs_points_per_slab (grid-point time derivatives per slab after the
        start-up) and launches_per_slab."""
        r, t, p, n = ctypes.c_int(), _I64(), _I64(), ctypes.c_int()
        _check(lib().dgsw_adams_info(self._h, ctypes.byref(r), ctypes.byref(t), ctypes.byref(p),
                                     ctypes.byref(n)), self._h)
        return {"ring_slots": r.value, "ticks_per_slab": t.value,
                "rhs_points_per_slab": p.value, "launches_per_slab": n.value}

    def synchronize(self):
        _check(lib().dgsw_synchronize(self._h), self._h)

    # state ---------------------------------------------------------------
    def set_state(self, u):
        """u: numpy float64 host array or torch float64 tensor (host or cuda)."""
        if hasattr(u, "is_cuda") and u.is_cuda:
            _torch_ready(u)
            _check(lib().dgsw_set_state_device(self._h, _ptr(u)), self._h)
            self.synchronize()
        else:
            a = u if isinstance(u, np.ndarray) else u.numpy()
            a = np.ascontiguousarray(a, dtype=np.float64)
            assert a.size == self.state_size
            _check(lib().dgsw_set_state(self._h, _ptr(a)), self._h)
            self.synchronize()

    def get_state(self, out=None):
        if out is not None and hasattr(out, "is_cuda") and out.is_cuda:
            _torch_ready(out)
            _check(lib().dgsw_get_state_device(self._h, _ptr(out)), self._h)
            self.synchronize()
            return out
        a = np.empty(self.state_size) if out is None else out
        _check(lib().dgsw_get_state(self._h, _ptr(a)), self._h)
        return a

    def set_initial_data(self, kind: str, params, t: float = 0.0):
        k = {"plane_wave": 0, "gaussian": 1, "gaussian_shell": 2}[kind]
        p = np.ascontiguousarray(params, dtype=np.float64).ravel()
        _check(lib().dgsw_set_initial_data(self._h, k, _ptr(p), float(t)), self._h)

    # TimeDerivative + BoundaryCorrection --------------------------------
    def rhs(self, u):
        """du/dt of a host state (numpy) or device state (torch cuda)."""
        if hasattr(u, "is_cuda") and u.is_cuda:
            import torch
            out = torch.empty_like(u)
            _torch_ready(u, out)
            _check(lib().dgsw_rhs_device(self._h, _ptr(u), _ptr(out)), self._h)
            self.synchronize()
            return out
        a = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty_like(a)
        _check(lib().dgsw_rhs(self._h, _ptr(a), _ptr(out)), self._h)
        return out

    def volume_rhs(self, u_dev):
        import torch
        out = torch.empty_like(u_dev)
        _torch_ready(u_dev, out)
        _check(lib().dgsw_volume_rhs_device(self._h, _ptr(u_dev), _ptr(out)), self._h)
        self.synchronize()
        return out

    # TimeStepper ---------------------------------------------------------
    def step(self, n_steps: int, dt: float, sync: bool = True):
        _check(lib().dgsw_step(self._h, int(n_steps), float(dt)), self._h)
        if sync:
            self.synchronize()

    def step_host(self, u, n_steps: int, dt: float):
        """n_steps on a host state (numpy float64, contiguous; pinned memory,
        e.g. a torch pin_memory tensor's numpy view, for full bandwidth),
        stepped in place: the copies overlap the first and last steps."""
        a = u if isinstance(u, np.ndarray) else u.numpy()
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] and a.size == self.state_size
        _check(lib().dgsw_step_host(self._h, _ptr(a), int(n_steps), float(dt)), self._h)
        return a

    def substep(self, k: int, dt: float):
        _check(lib().dgsw_substep(self._h, int(k), float(dt)), self._h)
        self.synchronize()

    def autotune(self, force_variant: int = -1):
        """Re-times the FP64 stage's launch variants on this handle; returns
        (chosen variant, [ms per launch of each]).  force_variant >= 0
        imposes a variant afterwards."""
        v = _I()
        ms = np.zeros(STAGE_VARIANTS)
        _check(lib().dgsw_autotune(self._h, int(force_variant), ctypes.byref(v), _ptr(ms)),
               self._h)
        return v.value, ms

    TUNE_FAMILIES = {0: "none", 1: "fp64_stage", 2: "mixed_batch", 3: "mixed_pipe",
                     4: "mixed_curved"}

    def tune(self, force_variant: int = -1):
        """Re-times the launch shapes of the handle's step kernels on its own
        state (dgsw_tune); returns {"family", "variant", "ms_per_step": [...]}
        with one time per candidate.  force_variant >= 0 imposes a shape."""
        fam, nv, v = _I(), _I(), _I()
        ms = np.zeros(8)
        _check(lib().dgsw_tune(self._h, int(force_variant), ctypes.byref(fam), ctypes.byref(nv),
                               ctypes.byref(v), _ptr(ms)), self._h)
        return {"family": self.TUNE_FAMILIES.get(fam.value, str(fam.value)),
                "variant": v.value, "ms_per_step": [float(x) for x in ms[:nv.value]]}

    def check_device_timeout(self, limit_seconds: float = 0.05) -> int:
        """Runs the bounded device wait on a barrier nothing completes; returns
        the status (DGSW_ERR_DEVICE_TIMEOUT when the wait gave up)."""
        return lib().dgsw_check_device_timeout(self._h, float(limit_seconds))

    NORM_NAMES = ("Max", "Min", "L2Norm", "L2IntegralNorm", "VolumeIntegral")
    VARIABLE_NAMES = ("Psi", "Pi", "Phi_x", "Phi_y", "Phi_z")

    def observe_norms(self, u_dev=None, subtract_dev=None):
        """Events::ObserveNorms of the state (or of a device tensor): a dict
        {"Max(Psi)": ..., ..., "NumberOfPoints": ..., "Volume": ...}."""
        out = np.zeros(27)
        _torch_ready(u_dev, subtract_dev)
        _check(lib().dgsw_observe_norms(self._h, _ptr(u_dev), _ptr(subtract_dev), _ptr(out)),
               self._h)
        return self._norm_dict(out)

    def observe_plane_wave_errors(self, k, t: float):
        """ObserveNorms of Psi - PlaneWave(k, t) etc. (the Error(...) norms)."""
        kk = np.ascontiguousarray(k, dtype=np.float64)
        out = np.zeros(27)
        _check(lib().dgsw_observe_plane_wave_errors(self._h, _ptr(kk), float(t), _ptr(out)),
               self._h)
        return self._norm_dict(out, prefix="Error")

    def _norm_dict(self, out, prefix=""):
        d = {}
        for v, vn in enumerate(self.VARIABLE_NAMES):
            name = "%s(%s)" % (prefix, vn) if prefix else vn
            for m, mn in enumerate(self.NORM_NAMES):
                d["%s(%s)" % (mn, name)] = float(out[5 * v + m])
        d["NumberOfPoints"] = int(out[25])
        d["Volume"] = float(out[26])
        d["raw"] = out
        return d

    def set_exponential_filter(self, alpha: float, half_power: int, enable: bool = True):
        """Filters::Exponential after every substep (dg::Actions::Filter)."""
        _check(lib().dgsw_set_exponential_filter(self._h, float(alpha), int(half_power),
                                                 1 if enable else 0), self._h)

    # discrete adjoint -----------------------------------------------------
    def adjoint_rhs(self, lam_dev):
        """L^T lambda (device tensors)."""
        import torch
        out = torch.empty_like(lam_dev)
        _torch_ready(lam_dev, out)
        _check(lib().dgsw_adjoint_rhs_device(self._h, _ptr(lam_dev), _ptr(out)), self._h)
        self.synchronize()
        return out

    def adjoint_autotune(self, force_variant: int = -1):
        """Re-times the adjoint kernel's two work splits on this handle;
        returns (chosen split, [ms per L^T launch of each]).  force_variant
        0 / 1 imposes a split afterwards."""
        v = _I()
        ms = np.zeros(2)
        _check(lib().dgsw_adjoint_autotune(self._h, int(force_variant), ctypes.byref(v),
                                           _ptr(ms)), self._h)
        return v.value, ms

    def set_samples(self, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.n_samples = a.shape[0]
        _check(lib().dgsw_set_samples(self._h, a.shape[0], _ptr(a)), self._h)

    def sample_psi(self):
        out = np.empty(self.n_samples)
        _check(lib().dgsw_sample_psi(self._h, _ptr(out)), self._h)
        return out

    def misfit_forward(self, targets, steps_per_window: int, dt: float) -> float:
        t = np.ascontiguousarray(targets, dtype=np.float64)
        n_windows = t.shape[0]
        J = ctypes.c_double()
        _check(lib().dgsw_misfit_forward(self._h, n_windows, int(steps_per_window), float(dt),
                                         _ptr(t), ctypes.byref(J)), self._h)
        return J.value

    def misfit_adjoint(self):
        """dJ/du(t=0) of the last misfit_forward, as a device tensor."""
        import torch
        g = torch.empty(self.state_size, dtype=torch.float64, device="cuda:%d" % self.device)
        _torch_ready(g)
        _check(lib().dgsw_misfit_adjoint(self._h, _ptr(g)), self._h)
        return g


class CurvedDgEvolution(DgEvolution):
    """The CurvedScalarWave DG step (EvolveCurvedScalarWave's ComputeTimeDerivative
    + ApplyBoundaryCorrections + UpdateU) on a Shell, one handle on one GPU.
    gamma2 is CurvedScalarWave's constraint damping gamma2."""

    def __init__(self, shell: Shell, points: int, precision=PRECISION_FP64, gamma2=1.0,
                 device=0, time_stepper="rk3_hesthaven_ssp", order=3, step_levels=None):
        """time_stepper "adams_bashforth": the stepper family the reference's
        curved executable runs (AdamsBashforth with local time stepping);
        FP64 only."""
        super().__init__(shell, points, precision, gamma2, device, time_stepper=time_stepper,
                         order=order, step_levels=step_levels)
        self.shell = shell

    def set_gaussian_shell(self, amplitude=1.0, radius=8.0, width=1.0):
        self.set_initial_data("gaussian_shell", [amplitude, radius, width])
