"""ctypes binding of the rigc C ABI (include/rigc.h).

The CUDA library is the only compute path: if ``librigc.so`` cannot be found
or loaded, importing the binding raises.  Device pointers come from torch
CUDA tensors (``tensor.data_ptr()``); results in device memory are copied out
with ``rigc_copy``.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "librigc.so")

RIGC_OK = 0
RIGC_ERR_ARG = 1
RIGC_ERR_CUDA = 2
RIGC_ERR_OOM = 3
RIGC_ERR_QUEUE_OVERFLOW = 4
RIGC_ERR_ITER_LIMIT = 5
RIGC_ERR_NAN = 6

RIGC_GRAD = 1
RIGC_HESS = 2
RIGC_PROJECT_PSD = 4
RIGC_TOI_NO_PRUNE = 1

EXPORTS = [
    "rigc_ctx_create", "rigc_ctx_destroy", "rigc_set_stream", "rigc_status_string",
    "rigc_get_stats", "rigc_copy", "rigc_world_vertices", "rigc_detect_candidates",
    "rigc_earliest_toi", "rigc_compute_earliest_toi", "rigc_construct_constraint_set",
    "rigc_set_constraints", "rigc_barrier_term", "rigc_barrier_local_terms",
    "rigc_narrow_phase_host", "rigc_barrier_local_terms_noalloc", "rigc_body_energy",
    "rigc_friction_setup", "rigc_get_friction", "rigc_friction_term", "rigc_friction_local_terms",
    "rigc_set_candidates", "rigc_set_ccd_budget", "rigc_sim_init", "rigc_sim_step",
    "rigc_sim_get_state", "rigc_ctx_create_batched", "rigc_num_scenes", "rigc_scene_tois",
    "rigc_scene_barrier_energies", "rigc_sim_rollout", "rigc_sim_backward",
    "rigc_sim_scene_params", "rigc_autotune", "rigc_set_tune", "rigc_fp64_throughput",
    "rigc_min_distance", "rigc_detect_intersections", "rigc_earliest_toi_piecewise_linear",
    "rigc_compute_earliest_toi_piecewise_linear", "rigc_set_pl_search", "rigc_set_ccd_window",
    "rigc_sim_set_kinematic",
]
RIGC_ERR_TOO_LARGE = 7
RIGC_ERR_SOLVE = 8
RIGC_NOALLOC_MAX_BODIES = 4096

_vp = C.c_void_p
_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)


class SceneDesc(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_int32), ("num_vertices", C.c_int32),
        ("num_edges", C.c_int32), ("num_faces", C.c_int32),
        ("rest_vertices", _d), ("edges", _i32), ("faces", _i32),
        ("faces_to_edges", _i32), ("body_vertex_start", _i32),
        ("body_edge_start", _i32), ("body_face_start", _i32),
        ("group_ids", _i32), ("body_types", _i32), ("r_max", _d),
        ("average_edge_length", C.c_double),
    ]


class Candidates(C.Structure):
    _fields_ = [("num_ee", C.c_int64), ("num_fv", C.c_int64), ("ee", _vp), ("fv", _vp)]


class ConstraintsView(C.Structure):
    _fields_ = [("num", C.c_int64), ("num_vv", C.c_int64), ("num_ev", C.c_int64),
                ("num_ee", C.c_int64), ("num_fv", C.c_int64), ("type", _vp), ("verts", _vp),
                ("prims", _vp), ("bodies", _vp), ("weight", _vp), ("eps_x", _vp)]


class BodyState(C.Structure):
    _fields_ = [("mass", _vp), ("moment", _vp), ("x_t0", _vp), ("v_t0", _vp),
                ("Qdot_t0", _vp), ("dof_fixed", _vp)]


class BarrierOut(C.Structure):
    _fields_ = [("energy", C.c_double), ("nnzb", C.c_int64), ("grad", _vp),
                ("row_ptr", _vp), ("col", _vp), ("val", _vp)]


class FrictionView(C.Structure):
    _fields_ = [("num", C.c_int64), ("mu", C.c_double), ("type", _vp), ("verts", _vp),
                ("bodies", _vp), ("coef", _vp)]


class SimParams(C.Structure):
    _fields_ = [("timestep", C.c_double), ("gravity", C.c_double * 3), ("dhat", C.c_double),
                ("dmin", C.c_double), ("coefficient_friction", C.c_double),
                ("static_friction_speed_bound", C.c_double), ("max_newton_iterations", C.c_int32),
                ("velocity_conv_tol", C.c_double), ("velocity_conv_tol_abs", C.c_int32),
                ("line_search_lower_bound", C.c_double), ("dhat_epsilon", C.c_double),
                ("min_barrier_stiffness_scale", C.c_double), ("average_mass", C.c_double),
                ("world_bbox_diagonal", C.c_double), ("newton_polish", C.c_int32),
                ("ccd_rescale", C.c_double), ("trajectory_type", C.c_int32)]


class SimState(C.Structure):
    _fields_ = [("mass", _vp), ("moment", _vp), ("dof_fixed", _vp), ("poses", _vp),
                ("velocities", _vp), ("Qdot", _vp)]


class TuneReport(C.Structure):
    _fields_ = [("ccd_blocks_per_sm", C.c_int32), ("cache_slots_per_body", C.c_int32),
                ("barrier_per_warp", C.c_int32), ("ccd_ms_default", C.c_double),
                ("ccd_ms", C.c_double), ("barrier_ms_default", C.c_double),
                ("barrier_ms", C.c_double), ("ccd_seeds_log2", C.c_int32),
                ("ccd_hand_off", C.c_int32), ("ccd_warp", C.c_int32),
                ("ccd_window_log2", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("newton_iterations", C.c_int64), ("newton_steps", C.c_int64),
                ("objective_evals", C.c_int64), ("ccd_calls", C.c_int64),
                ("cg_iterations", C.c_int64), ("barrier_stiffness", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("ccd_boxes", C.c_int64), ("ccd_candidates", C.c_int64),
                ("ccd_collisions", C.c_int64), ("grid_items", C.c_int64),
                ("large_elements", C.c_int64), ("cand_ee", C.c_int64),
                ("cand_fv", C.c_int64), ("kernel_launches", C.c_int64),
                ("last_status", C.c_int32), ("ccd_launches", C.c_int32),
                ("ccd_pieces", C.c_int64)]


_lib = None


def load():
    """Load librigc.so (built by rigid-ipc_gb300/build.py); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"rigc CUDA library not built ({LIB_PATH}); run rigid-ipc_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    L.rigc_ctx_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(_vp)]
    L.rigc_ctx_destroy.argtypes = [_vp]
    L.rigc_set_stream.argtypes = [_vp, _vp]
    L.rigc_status_string.restype = C.c_char_p
    L.rigc_status_string.argtypes = [C.c_int]
    L.rigc_get_stats.argtypes = [_vp, C.POINTER(Stats)]
    L.rigc_copy.argtypes = [_vp, _vp, _vp, C.c_size_t]
    L.rigc_world_vertices.argtypes = [_vp, _vp, _vp]
    L.rigc_detect_candidates.argtypes = [_vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(Candidates)]
    L.rigc_earliest_toi.argtypes = [_vp, _vp, _vp, C.c_double, C.c_int, _d, _vp]
    L.rigc_compute_earliest_toi.argtypes = [_vp, _vp, _vp, C.c_double, _d]
    L.rigc_earliest_toi_piecewise_linear.argtypes = [_vp, _vp, _vp, C.c_double, _d, _vp]
    L.rigc_compute_earliest_toi_piecewise_linear.argtypes = [_vp, _vp, _vp, C.c_double, _d]
    L.rigc_set_pl_search.argtypes = [_vp, C.c_int32]
    L.rigc_set_ccd_window.argtypes = [_vp, C.c_int32]
    L.rigc_sim_set_kinematic.argtypes = [_vp, C.c_int32, C.c_double, C.c_int64, _vp]
    L.rigc_construct_constraint_set.argtypes = [_vp, _vp, C.c_double, C.c_double,
                                                C.POINTER(ConstraintsView)]
    L.rigc_set_constraints.argtypes = [_vp, C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp]
    L.rigc_barrier_term.argtypes = [_vp, _vp, C.c_double, C.c_double, C.c_int,
                                    C.POINTER(BarrierOut)]
    L.rigc_barrier_local_terms.argtypes = [_vp, _vp, C.c_double, C.c_double, C.c_int, _vp, _vp, _vp]
    L.rigc_narrow_phase_host.argtypes = [_vp, _vp, _vp, C.c_double, C.c_double, _d, _d, _vp, _vp,
                                         _vp, _vp, C.c_int64, _i64]
    L.rigc_body_energy.argtypes = [_vp, C.POINTER(BodyState), _vp, _d, C.c_double, _d, _vp, _vp]
    L.rigc_fp64_throughput.argtypes = [C.c_int32, C.c_int32, C.c_int32, _d, _d, _d]
    L.rigc_min_distance.argtypes = [_vp, _vp, C.c_double, C.c_double, _d]
    L.rigc_detect_intersections.argtypes = [_vp, _vp, _i64]
    L.rigc_barrier_local_terms_noalloc.argtypes = [
        _vp, C.c_int64, C.c_int32, _vp, C.c_int64, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_double,
        C.c_int, _vp, _vp, _vp, _vp]
    L.rigc_friction_setup.argtypes = [_vp, _vp, C.c_double, C.c_double, C.c_double, _i64]
    L.rigc_get_friction.argtypes = [_vp, C.POINTER(FrictionView)]
    L.rigc_friction_term.argtypes = [_vp, _vp, C.c_double, C.c_int, C.POINTER(BarrierOut)]
    L.rigc_friction_local_terms.argtypes = [_vp, _vp, C.c_double, C.c_int, _vp, _vp, _vp]
    L.rigc_set_candidates.argtypes = [_vp, C.c_int64, _vp, C.c_int64, _vp]
    L.rigc_set_ccd_budget.argtypes = [_vp, C.c_int64]
    L.rigc_sim_init.argtypes = [_vp, C.POINTER(SimParams), C.POINTER(SimState)]
    L.rigc_sim_step.argtypes = [_vp, C.c_int32, C.POINTER(StepStats)]
    L.rigc_sim_get_state.argtypes = [_vp, _vp, _vp, _vp, _d]
    L.rigc_sim_rollout.argtypes = [_vp, C.c_int32, C.c_int32, C.POINTER(StepStats)]
    L.rigc_sim_backward.argtypes = [_vp] + [_vp] * 6
    L.rigc_sim_scene_params.argtypes = [_vp, _vp, _vp]
    L.rigc_autotune.argtypes = [_vp, _vp, _vp, C.c_double, C.c_double, C.POINTER(TuneReport)]
    L.rigc_set_tune.argtypes = [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.rigc_ctx_create_batched.argtypes = [C.POINTER(SceneDesc), C.c_int32, _vp, C.POINTER(_vp)]
    L.rigc_num_scenes.argtypes = [_vp]
    L.rigc_scene_tois.argtypes = [_vp, _d]
    L.rigc_scene_barrier_energies.argtypes = [_vp, _d]
    for f in EXPORTS:
        getattr(L, f).restype = C.c_char_p if f == "rigc_status_string" else C.c_int
    _lib = L
    return L


class RigcError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = load().rigc_status_string(status).decode()
        super().__init__(f"{where}: status {status} ({msg})")


def check(status, where, allow=()):
    if status != RIGC_OK and status not in allow:
        raise RigcError(status, where)
    return status
