"""ctypes binding of the C ABI declared in include/p2de.h (libp2de_gpu.so).

The library is built in-tree (p2de.jl_gb300/_build). There is no CPU fallback:
loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_size_t, c_void_p
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "_build" / "libp2de_gpu.so"

# p2de_status
P2DE_OK = 0
STATUS_NAMES = {
    0: "P2DE_OK",
    1: "P2DE_ERR_INVALID_ARGUMENT",
    2: "P2DE_ERR_UNSUPPORTED",
    3: "P2DE_ERR_CUDA",
    4: "P2DE_ERR_OUT_OF_MEMORY",
    5: "P2DE_ERR_NOT_POSITIVE",
    6: "P2DE_ERR_BAD_DT",
    7: "P2DE_ERR_NO_DEVICE",
    8: "P2DE_ERR_BUDGET",
    9: "P2DE_ERR_NOT_FOUND",
}

# p2de_rhs_type
RHS_ES_LIMITED_LOW_ORDER_POS = 0
RHS_LOW_ORDER_POSITIVITY = 1
RHS_ENTROPY_STABLE = 2
# p2de_bound_type
BOUND_POSITIVITY = 0
BOUND_POSITIVITY_AND_CELL_ENTROPY = 1
BOUND_TVD = 2
BOUND_TVD_AND_CELL_ENTROPY = 3
BOUND_POSITIVITY_AND_MIN_ENTROPY = 4
BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY = 5
BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY = 6
BOUND_TVD_AND_MIN_ENTROPY = 7
BOUND_TVD_AND_RELAXED_MIN_ENTROPY = 8
BOUND_TVD_AND_RELAXED_CELL_ENTROPY = 9
# p2de_rhs_limiter
LIMITER_SUBCELL = 0
LIMITER_ZHANG_SHU = 1
# p2de_surface_flux
FLUX_LF_NODAL = 0
FLUX_LF_PROJECTED = 1
# p2de_precision
PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_MIXED_ACC64 = 2
PRECISIONS = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "mixed-acc64": PRECISION_MIXED_ACC64}
# p2de_field
FIELD_UQ = 0
FIELD_RHSU = 1
FIELD_RHSL = 2
FIELD_RHSH = 3
FIELD_RHSXYL = 4
FIELD_RHSXYH = 5
FIELD_BF_L = 6
FIELD_BF_H = 7
FIELD_L_LOCAL = 8
FIELD_RESW = 9
FIELD_L = 10
FIELD_THETA_LOCAL = 11
LAYOUT_FLAT = 0  # p2de_layout
LAYOUT_LINES_PER_WARP = 1
LAYOUT_TEAM = 2  # Line solves: a team of lanes per element
FIELD_F_BAR_H = 12  # f_bar_H of the last limited stage: 2 x (Nq+N1D) x K states, x then y
FIELD_F_BAR_L = 13
# p2de_equation
EQUATION_COMPRESSIBLE_EULER = 0
EQUATION_KPP = 1
EQUATION_COMPRESSIBLE_EULER_1D = 2
# p2de_basis, p2de_entropyproj_limiter
BASIS_LOBATTO = 0
BASIS_GAUSS = 1
ENTROPYPROJ_NONE = 0
ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION = 1


class P2deParam(ctypes.Structure):
    _fields_ = [
        ("N", c_int32),
        ("K", c_int32),
        ("gamma", c_double),
        ("POSTOL", c_double),
        ("ZEROTOL", c_double),
        ("zeta", c_double),
        ("eta", c_double),
        ("CFL", c_double),
        ("dt0", c_double),
        ("t0", c_double),
        ("T", c_double),
        ("rhs_type", c_int32),
        ("bound_type", c_int32),
        ("low_order_surface_flux", c_int32),
        ("high_order_surface_flux", c_int32),
        ("reference_semantics", c_int32),
        ("precision", c_int32),
        ("shock_capture", c_int32),
        ("rhs_limiter", c_int32),
        ("shock_capture_a", c_double),
        ("shock_capture_c", c_double),
        ("bound_beta", c_double),
        ("approximation_basis", c_int32),
        ("entropyproj_limiter", c_int32),
        ("equation", c_int32),
        ("reserved_", c_int32),
    ]


class P2deMesh(ctypes.Structure):
    _fields_ = [
        ("geom", POINTER(c_double)),
        ("mapP", POINTER(c_int64)),
        ("mapI", POINTER(c_int64)),
        ("nI", c_int64),
        ("Ival", POINTER(c_double)),
        ("mapO", POINTER(c_int64)),
        ("nO", c_int64),
        ("mapW", POINTER(c_int64)),
        ("nW", c_int64),
        ("mapS", POINTER(c_int64)),
        ("nS", c_int64),
        ("xyS", POINTER(c_double)),
        ("shock_x0", c_double),
        ("shock_inv_slope", c_double),
        ("shock_speed", c_double),
        ("shock_post", c_double * 4),
        ("shock_pre", c_double * 4),
    ]


class P2deDeviceMesh(ctypes.Structure):
    """p2de_device_mesh: device pointers for p2de_rhs_noalloc."""

    _fields_ = [
        ("geom", c_void_p),
        ("nbr", c_void_p),
        ("bc", c_void_p),
        ("bcidx", c_void_p),
        ("Ival", c_void_p),
        ("nI", c_int64),
        ("xyS", c_void_p),
        ("nS", c_int64),
        ("shock_x0", c_double),
        ("shock_inv_slope", c_double),
        ("shock_speed", c_double),
        ("shock_post", c_double * 4),
        ("shock_pre", c_double * 4),
        ("axis_aligned", c_int32),
    ]


class P2deError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# (name, restype, argtypes) of every entry point in include/p2de.h
SOLVER_P = c_void_p
EXPORTS = [
    ("p2de_abi_version", c_int, []),
    ("p2de_solver_field_count", c_int, [SOLVER_P, c_int32, POINTER(c_int64)]),
    ("p2de_field_count", c_int, [c_int32, c_int32, c_int32, POINTER(c_int64)]),
    ("p2de_initialize_DG", c_int, [POINTER(P2deParam), POINTER(P2deMesh), c_int, POINTER(c_void_p)]),
    ("p2de_destroy", c_int, [SOLVER_P]),
    ("p2de_set_Uq", c_int, [SOLVER_P, POINTER(c_double)]),
    ("p2de_get_field", c_int, [SOLVER_P, c_int32, c_int32, POINTER(c_double)]),
    ("p2de_rhs", c_int, [SOLVER_P, c_double, c_double, c_int32, POINTER(c_double)]),
    ("p2de_ssp33_step", c_int, [SOLVER_P, POINTER(c_double), POINTER(c_double)]),
    ("p2de_ssp33", c_int, [SOLVER_P, POINTER(c_double), POINTER(c_int64), POINTER(c_double)]),
    ("p2de_ssp33_advance", c_int, [SOLVER_P, c_int64, POINTER(c_double), POINTER(c_int64)]),
    ("p2de_device_ptr", c_int, [SOLVER_P, c_int32, POINTER(c_void_p)]),
    ("p2de_set_stream", c_int, [SOLVER_P, c_void_p]),
    ("p2de_launch_count", c_int, [SOLVER_P, POINTER(c_int64)]),
    ("p2de_min_rho_rhoe", c_int, [SOLVER_P, POINTER(c_double), POINTER(c_double)]),
    ("p2de_stage_minima", c_int, [SOLVER_P, POINTER(c_double)]),
    ("p2de_profile_steps", c_int, [SOLVER_P, c_int64, POINTER(c_double), POINTER(c_double)]),
    ("p2de_read_counters", c_int, [SOLVER_P, POINTER(ctypes.c_uint64), c_int32]),
    ("p2de_check_conservation", c_int, [SOLVER_P, POINTER(c_double), POINTER(c_double)]),
    ("p2de_calculate_error", c_int, [SOLVER_P, POINTER(c_double), POINTER(c_double)]),
    ("p2de_set_elements_per_block", c_int, [SOLVER_P, c_int32]),
    ("p2de_get_elements_per_block", c_int, [SOLVER_P, POINTER(c_int32), POINTER(c_int32)]),
    ("p2de_set_layout", c_int, [SOLVER_P, c_int32]),
    ("p2de_get_layout", c_int, [SOLVER_P, POINTER(c_int32)]),
    ("p2de_set_threads_per_block", c_int, [SOLVER_P, c_int32]),
    ("p2de_get_threads_per_block", c_int, [SOLVER_P, POINTER(c_int32)]),
    ("p2de_autotune", c_int, [SOLVER_P, POINTER(c_int32), POINTER(c_double)]),
    ("p2de_batch_create", c_int, [c_int, c_int32, c_size_t, c_int32, POINTER(c_void_p)]),
    ("p2de_batch_destroy", c_int, [c_void_p]),
    ("p2de_batch_solve_bytes", c_int, [POINTER(P2deParam), c_int64, c_int64, POINTER(c_size_t)]),
    ("p2de_batch_add", c_int, [c_void_p, POINTER(P2deParam), POINTER(P2deMesh), POINTER(c_double), POINTER(c_int32)]),
    ("p2de_batch_remove", c_int, [c_void_p, c_int32]),
    ("p2de_batch_step", c_int, [c_void_p, c_int64]),
    (
        "p2de_batch_state",
        c_int,
        [c_void_p, c_int32, POINTER(c_double), POINTER(c_double), POINTER(c_int64), POINTER(c_int32), POINTER(c_int32)],
    ),
    ("p2de_batch_states", c_int, [c_void_p, POINTER(c_double)]),
    ("p2de_batch_get_Uq", c_int, [c_void_p, c_int32, POINTER(c_double)]),
    ("p2de_batch_memory", c_int, [c_void_p, POINTER(c_size_t), POINTER(c_size_t)]),
    ("p2de_batch_launch_count", c_int, [c_void_p, POINTER(c_int64)]),
    ("p2de_batch_last_error", c_int, [c_void_p, c_char_p, c_size_t]),
    ("p2de_batch_set_elements_per_block", c_int, [c_void_p, c_int32, c_int32]),
    ("p2de_batch_get_elements_per_block", c_int, [c_void_p, c_int32, POINTER(c_int32), POINTER(c_int32)]),
    ("p2de_batch_set_layout", c_int, [c_void_p, c_int32, c_int32]),
    ("p2de_batch_get_layout", c_int, [c_void_p, c_int32, POINTER(c_int32)]),
    ("p2de_batch_autotune", c_int, [c_void_p, POINTER(c_int32)]),
    ("p2de_server_create", c_int, [c_int, c_int32, c_size_t, c_int32, c_int32, POINTER(c_void_p)]),
    ("p2de_server_submit", c_int, [c_void_p, POINTER(P2deParam), POINTER(P2deMesh), POINTER(c_double), POINTER(c_int64)]),
    (
        "p2de_server_poll",
        c_int,
        [c_void_p, c_int64, POINTER(c_int32), POINTER(c_double), POINTER(c_double), POINTER(c_int64)],
    ),
    ("p2de_server_wait", c_int, [c_void_p, c_int64, c_double, POINTER(c_int32)]),
    ("p2de_server_result", c_int, [c_void_p, c_int64, POINTER(c_double)]),
    ("p2de_server_stats", c_int, [c_void_p, POINTER(c_double)]),
    ("p2de_server_destroy", c_int, [c_void_p]),
    ("p2de_noalloc_max_elements", c_int, [c_int32, POINTER(c_int64)]),
    (
        "p2de_rhs_noalloc",
        c_int,
        [POINTER(P2deParam), POINTER(P2deDeviceMesh), c_void_p, c_double, c_double, c_int32, c_void_p, POINTER(c_double), c_void_p],
    ),
    ("p2de_last_error", c_int, [SOLVER_P, c_char_p, c_size_t]),
]

_LIB = None


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads libp2de_gpu.so and declares every export. Raises when it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python p2de.jl_gb300/build.py` "
            "(there is no CPU fallback for the GPU path)"
        )
    lib = ctypes.CDLL(str(p))
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def last_error(lib, handle) -> str:
    buf = ctypes.create_string_buffer(1024)
    lib.p2de_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(lib, status: int, handle=None) -> None:
    if status != P2DE_OK:
        raise P2deError(status, last_error(lib, handle))


def dptr(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_int64))
