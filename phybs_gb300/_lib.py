"""ctypes binding of libphybs_gb300.so (the C ABI declared in include/phybs.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly if the shared library was not built (run ``build()`` of
``__graft_entry__`` or ``python -m phybs_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

PBS_OK = 0
PBS_E_INVALID_ARG = -1
PBS_E_CUDA = -2
PBS_E_NONFINITE = -3
PBS_E_ITER_CAP = -4
PBS_E_BAD_MESH = -5
PBS_E_NO_DEVICE = -6
PBS_E_OUT_OF_MEMORY = -7
PBS_E_CAPACITY = -8
PBS_E_DEVICE_TIMEOUT = -9

PBS_MATERIAL_NEOHOOKEAN = 0
PBS_MATERIAL_STRETCH = 1
PBS_CONTROL_REFERENCE = 0
PBS_CONTROL_RESTART = 1
PBS_CLAMP_CPU = 0
PBS_CLAMP_GPU = 1
PBS_ENGINE_GRAPH = 0
PBS_ENGINE_FRAME = 1

# Every entry point include/phybs.h declares.
EXPORTS = (
    "pbs_default_params", "pbs_error_string", "pbs_create", "pbs_destroy", "pbs_lame", "pbs_set_material",
    "pbs_set_params", "pbs_get_params", "pbs_step", "pbs_read_positions", "pbs_update_positions",
    "pbs_read_velocities", "pbs_write_velocities", "pbs_reset", "pbs_get_stats", "pbs_get_sizes",
    "pbs_get_incidence", "pbs_get_rest_data", "pbs_eval_tets", "pbs_eval_nodes", "pbs_stiffness_pattern",
    "pbs_set_node_positions", "pbs_get_stream", "pbs_profile_kernels",
    "pbs_mlp_param_count", "pbs_mlp_create", "pbs_mlp_destroy", "pbs_mlp_get_params", "pbs_mlp_set_params",
    "pbs_mlp_forward", "pbs_mlp_gradient", "pbs_mlp_set_data", "pbs_mlp_train",
    "pbs_set_warm_start", "pbs_warm_start_features", "pbs_eval_nodes_static",
    "pbs_set_surface", "pbs_get_face_ring", "pbs_pick_face", "pbs_drag_face_ring", "pbs_backward_euler_step",
    "pbs_set_guess", "pbs_autotune", "pbs_get_instance_stats", "pbs_set_chunk_shape",
    "pbs_pbd_step", "pbs_pd_step", "pbs_eval_fp64_svd_count",
    "pbs_set_pass_engine", "pbs_get_pass_engine", "pbs_profile_frame", "pbs_eval_base_force",
    "pbs_set_l2_residency",
)

PBS_EVAL_STATIC_MAX_TETS = 524288


class MeshDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("rest", C.c_void_p), ("positions", C.c_void_p), ("n_tets", C.c_int),
                ("tets", C.c_void_p), ("pin_mask", C.c_void_p), ("n_instances", C.c_int),
                ("instance_node_ptr", C.c_void_p), ("instance_tet_ptr", C.c_void_p), ("density", C.c_float),
                ("gravity", C.c_float)]


class StepParams(C.Structure):
    _fields_ = [("h", C.c_float), ("max_iters", C.c_int), ("tol", C.c_float), ("control", C.c_int),
                ("alpha0", C.c_float), ("alpha_min", C.c_float), ("alpha_shrink", C.c_float),
                ("line_search_every", C.c_int), ("hessian_every", C.c_int), ("n_profile", C.c_int),
                ("profile_k", C.c_int * 4), ("profile_rho", C.c_float * 4), ("damping", C.c_float),
                ("warm_start", C.c_float), ("body_force_scale", C.c_float), ("energy_clamp", C.c_int),
                ("pass_cap", C.c_int), ("energy_slack", C.c_float), ("alpha_grow", C.c_float),
                ("incremental_stress", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("passes", C.c_int), ("iterations", C.c_int), ("rejections", C.c_int), ("converged", C.c_int),
                ("status", C.c_int), ("alpha", C.c_float), ("rho", C.c_float), ("omega", C.c_float),
                ("energy", C.c_double), ("residual_ratio", C.c_double), ("device_ms", C.c_double),
                ("graph_launches", C.c_int), ("warm_start_used", C.c_int), ("guess_fallbacks", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("chunk_threads", C.c_int), ("chunk_tets", C.c_int), ("chunk_nodes", C.c_int),
                ("chunk_staged", C.c_int), ("node_npt", C.c_int), ("n_tried", C.c_int),
                ("pass_ms", C.c_double), ("default_pass_ms", C.c_double)]


class PhybsError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__(f"{what}: {error_string(code)} ({code})" if what else f"{error_string(code)} ({code})")


_lib = None


def lib():
    """Load the library (raises OSError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise OSError(f"{LIB} is missing: build the CUDA extension first")
        L = C.CDLL(LIB)
        L.pbs_error_string.restype = C.c_char_p
        L.pbs_destroy.restype = None
        L.pbs_default_params.restype = None
        L.pbs_lame.restype = None
        _lib = L
    return _lib


def error_string(code: int) -> str:
    try:
        return lib().pbs_error_string(C.c_int(code)).decode()
    except OSError:
        return f"error {code}"


def check(code: int, what: str = "") -> int:
    if code != PBS_OK:
        raise PhybsError(code, what)
    return code


def default_params() -> StepParams:
    p = StepParams()
    lib().pbs_default_params(C.byref(p))
    return p


def lame(young: float, poisson: float, reference_formula: bool = True):
    mu, lam = C.c_float(), C.c_float()
    lib().pbs_lame(C.c_float(young), C.c_float(poisson), C.c_int(1 if reference_formula else 0), C.byref(mu),
                   C.byref(lam))
    return mu.value, lam.value
