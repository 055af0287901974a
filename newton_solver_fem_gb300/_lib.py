"""ctypes binding of ``libfemgb300.so`` (declarations mirror ``include/fem_gb300.h``).

The library is required: loading fails loudly when it has not been built, and
there is no CPU fallback for the solver path.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIBRARY = Path(__file__).resolve().with_name("libfemgb300.so")

FEM_OK = 0
FEM_ERR_BAD_ARG = 1
FEM_ERR_NOT_CONVERGED = 2
FEM_ERR_NON_FINITE = 3
FEM_ERR_TIMEOUT = 4
FEM_ERR_CUDA = 5
FEM_ERR_UNSUPPORTED = 6

FEM_PRECOND_BLOCK_DIAG = 0
FEM_PRECOND_DIAG = 1

FEM_TUNE_SPMV_UNROLL = 1
FEM_TUNE_L2_RESIDENT_BYTES = 2
FEM_TUNE_RESIDENT_SLICES = 3
FEM_TUNE_GRID = 4
FEM_TUNE_CTA_THREADS = 5
FEM_TUNE_GRID_CAP = 6
FEM_TUNE_RESIDENT_STATE = 7
FEM_TUNE_BALANCE = 8
FEM_TUNE_RESIDENT_LAYOUT = 9
FEM_TUNE_SPLIT_HEADROOM = 10
FEM_TUNE_TAIL_PREFETCH = 11
FEM_TUNE_COMPACT_COLUMNS = 12
FEM_TUNE_UNIFORM_COLUMN_BLOCKS = 13
FEM_TUNE_CG_VARIANT = 14
FEM_TUNE_OPERATOR_BATCH = 15
FEM_TUNE_OPERATOR_STAGE = 16

FEM_TERM_SPRING = 1
FEM_TERM_TET = 2
FEM_TERM_HEX = 4
FEM_TERM_GROUND = 8
FEM_TERM_GRAVITY = 16
FEM_TERM_DAMPING = 32
FEM_TERM_TRI = 64
FEM_TERM_PARTICLE = 128
FEM_TERM_SOFT_CONTACT = 256
FEM_TERM_SURFACE = 512
FEM_TERM_ALL = 1023

_f = ctypes.c_float
_i32 = ctypes.c_int32
_p = ctypes.c_void_p


class FemDesc(ctypes.Structure):
    _fields_ = [
        ("particle_count", _i32),
        ("tet_count", _i32),
        ("hex_count", _i32),
        ("spring_count", _i32),
        ("particle_q", _p),
        ("particle_mass", _p),
        ("particle_inv_mass", _p),
        ("particle_radius", _p),
        ("particle_flags", _p),
        ("tet_indices", _p),
        ("tet_poses", _p),
        ("tet_materials", _p),
        ("hex_indices", _p),
        ("hex_materials", _p),
        ("hex_inv_J0", _p),
        ("hex_det_J0_w", _p),
        ("spring_indices", _p),
        ("spring_rest_length", _p),
        ("spring_stiffness", _p),
        ("spring_damping", _p),
        ("fixed_indices", _p),
        ("fixed_count", _i32),
        ("scene_offsets", _p),
        ("scene_count", _i32),
        ("gravity", _f * 3),
        ("dt", _f),
        ("min_stretch", _f),
        ("max_stretch", _f),
        ("has_ground", _i32),
        ("ground_plane", _f * 4),
        ("ground_ke", _f),
        ("ground_kd", _f),
        ("ground_kf", _f),
        ("ground_mu", _f),
        ("linear_damping", _f),
        ("enable_tet_activations", _i32),
        ("preconditioner", _i32),
        ("maxiter", _i32),
        ("tolerance", _f),
        ("velocity_increment", _p),
        ("tri_count", _i32),
        ("tri_indices", _p),
        ("tri_poses", _p),
        ("tri_materials", _p),
        ("spring_rest_direction", _p),
        ("torque_stiffness", _f),
        ("torque_damping", _f),
        ("particle_contact", _i32),
        ("particle_ke", _f),
        ("particle_kd", _f),
        ("particle_kf", _f),
        ("particle_mu", _f),
        ("particle_cohesion", _f),
        ("particle_max_radius", _f),
        ("soft_contact_ke", _f),
        ("soft_contact_kd", _f),
        ("soft_contact_kf", _f),
        ("soft_contact_mu", _f),
    ]


class FemTopologyUpdate(ctypes.Structure):
    _fields_ = [(name, _i32) for name in (
        "dirty_elements", "removed_elements", "reused_elements", "active_elements", "touched_rows",
        "topology_inserted_elements", "topology_removed_elements", "full_numeric_refresh")]


class FemStats(ctypes.Structure):
    _fields_ = [
        ("status", _i32),
        ("scene_count", _i32),
        ("max_iterations", _i32),
        ("min_iterations", _i32),
        ("max_relative_residual", _f),
        ("unconverged_scenes", _i32),
        ("total_iterations", ctypes.c_int64),
    ]


class FemPreparedWs(ctypes.Structure):
    _fields_ = [(name, _p) for name in ("q", "v", "impulse", "predictor", "base_rhs", "increment", "diagonal")]


# (name, restype, argtypes) for every symbol declared in include/fem_gb300.h
SIGNATURES = [
    ("fem_create", _i32, [ctypes.POINTER(FemDesc), ctypes.POINTER(_p)]),
    ("fem_destroy", _i32, [_p]),
    ("fem_step", _i32, [_p, _p, _p, _p, _p, _p, _p, _p, _p, _f, _p]),
    ("fem_refresh_tangent", _i32, [_p, _p, _f, _p]),
    ("fem_refresh_topology", _i32, [_p, ctypes.POINTER(FemDesc), _p, _f, _p]),
    ("fem_rebuild_element_blocks", _i32, [_p, _p, _f, _p]),
    ("fem_refresh_preconditioner", _i32, [_p, _p]),
    ("fem_set_tolerance", _i32, [_p, _f]),
    ("fem_set_maxiter", _i32, [_p, _i32]),
    ("fem_set_wait_limit", _i32, [_p, ctypes.c_int64]),
    ("fem_set_tuning", _i32, [_p, _i32, ctypes.c_int64]),
    ("fem_get_tuning", _i32, [_p, _i32, ctypes.POINTER(ctypes.c_int64)]),
    ("fem_reset", _i32, [_p, _p]),
    ("fem_velocity_increment_ptr", _p, [_p]),
    ("fem_get_solve_residuals", _i32, [_p, _p, _i32, _p]),
    ("fem_get_stats", _i32, [_p, ctypes.POINTER(FemStats), _p, _p]),
    ("fem_set_soft_contacts", _i32, [_p, _p, _p, _p, _p, _p, _i32]),
    ("fem_set_surface_contacts", _i32, [_p, _i32, _p, _p, _p, _p, _f, _f, _p, _p]),
    ("fem_update_surface_contacts", _i32, [_p, _p, _p]),
    ("fem_set_timing", _i32, [_p, _i32]),
    ("fem_get_timing", _i32, [_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
    ("fem_eval_forces", _i32, [_p, _p, _p, _p, _p, _i32, _p, _p]),
    ("fem_matrix_info", _i32, [_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                               ctypes.POINTER(ctypes.c_int64)]),
    ("fem_export_bsr", _i32, [_p, _p, _p, _p, _p]),
    ("fem_export_preconditioner", _i32, [_p, _p, _p]),
    ("fem_export_triplets", _i32, [_p, _p, _p, _p, _p]),
    ("fem_set_mu_scale", _i32, [_p, _p]),
    ("fem_solve", _i32, [_p, _p, _p, _f, _i32, _p]),
    ("fem_force_vjp", _i32, [_p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    ("fem_predictor_vjp", _i32, [_p, _p, _f, _p, _p]),
    ("fem_force_vjp_materials", _i32, [_p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    ("fem_rollout_segment", _i32, [_p, _p, _p, _p, _i32, _p, _p, _p, _f, _f, _i32, _i32, _i32, _p, _p, _p, _p]),
    ("fem_adjoint_segment", _i32, [_p, _p, _p, _i32, _p, _p, _p, _f, _f, _i32, _i32, _p, _p, _p, _p, _p, _p, _p,
                                   _p, _p]),
    ("fem_prepare_tet_updates", _i32, [_p, ctypes.POINTER(FemDesc), _i32, _p]),
    ("fem_update_tet_topology", _i32, [_p, ctypes.POINTER(FemDesc), _p, _f, _p, ctypes.POINTER(FemTopologyUpdate),
                                        _p]),
    ("fem_prepare", _i32, [_p, ctypes.POINTER(FemPreparedWs), _p, _p, _p, _p, _p, _f, _p]),
    ("fem_prepared_rhs", _i32, [_p, ctypes.POINTER(FemPreparedWs), _p, _f, _p, _p]),
    ("fem_apply_operator", _i32, [_p, _p, _p, _p]),
    ("fem_apply_preconditioner", _i32, [_p, _p, _p, _p]),
    ("fem_prepared_solve", _i32, [_p, ctypes.POINTER(FemPreparedWs), _p, _f, _i32, _f, _p]),
    ("fem_prepared_reconstruct", _i32, [_p, ctypes.POINTER(FemPreparedWs), _p, _f, _p, _p, _p]),
    ("fem_pcg_solve_noalloc", _i32, [_p, _p, _p, _p, _p, _i32, _f, _i32, _p, _p]),
    ("fem_status_string", ctypes.c_char_p, [_i32]),
    ("fem_version", ctypes.c_char_p, []),
]

_LIB = None


def load() -> ctypes.CDLL:
    """Load the library once; raise if it has not been built."""
    global _LIB
    if _LIB is None:
        if not LIBRARY.exists():
            raise RuntimeError(
                f"{LIBRARY.name} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(or newton_solver_fem_gb300.build.build()) first"
            )
        lib = ctypes.CDLL(str(LIBRARY))
        for name, restype, argtypes in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _LIB = lib
    return _LIB


class FemError(RuntimeError):
    """A non-OK status from the native library."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def check(code: int, what: str = "") -> None:
    """Map a status code to the reference's exception types (ValueError / RuntimeError)."""
    if code == FEM_OK:
        return
    message = load().fem_status_string(code).decode()
    text = f"{what}: {message}" if what else message
    if code == FEM_ERR_BAD_ARG:
        raise ValueError(text)
    if code == FEM_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    raise FemError(code, text)
