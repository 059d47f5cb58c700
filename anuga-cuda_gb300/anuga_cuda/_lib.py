"""ctypes binding of libswgpu.so (declarations in include/swgpu.h).

The library is built in-tree by :func:`anuga_cuda._build.build`; importing
this module never falls back to anything else: if the shared library is
missing or cannot be loaded, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._build import library_path

__all__ = [
    "lib", "SwgpuError", "Mesh_t", "Params_t", "State_t", "BoundaryTag_t", "LaunchConfig_t",
    "check",
    "STAGE", "XMOMENTUM", "YMOMENTUM", "ELEVATION", "FRICTION", "HEIGHT", "XVELOCITY",
    "YVELOCITY", "FP64", "MIXED", "BC_REFLECTIVE", "BC_DIRICHLET", "BC_TIME_STAGE_SINE",
    "BC_TRANSMISSIVE", "BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM", "BC_INFLOW_HYDROGRAPH",
    "BC_TIME_STAGE_FOURIER",
    "STOP_NONE", "STOP_YIELD", "STOP_FINAL", "STOP_BUDGET", "STOP_ERROR", "EXPORTED_SYMBOLS",
    "EULER", "RK2", "RK3",
]

STAGE, XMOMENTUM, YMOMENTUM, ELEVATION, FRICTION, HEIGHT, XVELOCITY, YVELOCITY = range(8)
FP64, MIXED = 0, 1
EULER, RK2, RK3 = 1, 2, 3
BC_REFLECTIVE, BC_DIRICHLET, BC_TIME_STAGE_SINE = 0, 1, 2
BC_TRANSMISSIVE, BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM, BC_INFLOW_HYDROGRAPH = 3, 4, 5
BC_TIME_STAGE_FOURIER = 6
STOP_NONE, STOP_YIELD, STOP_FINAL, STOP_BUDGET, STOP_ERROR = range(5)

STATUS_NAMES = {
    0: "SWGPU_OK", 1: "SWGPU_EINVAL", 2: "SWGPU_ECUDA", 3: "SWGPU_ENOMEM",
    4: "SWGPU_EDENOMINATOR", 5: "SWGPU_ESMALLSTEP", 6: "SWGPU_ENONFINITE", 7: "SWGPU_EBED",
    8: "SWGPU_EBOUNDARY", 9: "SWGPU_EOVERSHOOT", 10: "SWGPU_EMESH", 11: "SWGPU_ETIMEOUT",
}

_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)


class Mesh_t(C.Structure):
    _fields_ = [
        ("number_of_elements", C.c_int64),
        ("number_of_boundary_elements", C.c_int64),
        ("neighbours", _i64p),
        ("neighbour_edges", _i64p),
        ("surrogate_neighbours", _i64p),
        ("number_of_boundaries", _i64p),
        ("tri_full_flag", _i64p),
        ("normals", _f64p),
        ("edgelengths", _f64p),
        ("radii", _f64p),
        ("areas", _f64p),
        ("vertex_coordinates", _f64p),
        ("centroid_coordinates", _f64p),
        ("boundary_cells", _i64p),
        ("boundary_edges", _i64p),
        ("boundary_tag", _i64p),
    ]


PARAM_FIELDS = [
    ("g", C.c_double), ("epsilon", C.c_double), ("H0", C.c_double),
    ("minimum_allowed_height", C.c_double), ("maximum_allowed_speed", C.c_double),
    ("beta_w", C.c_double), ("beta_w_dry", C.c_double), ("beta_uh", C.c_double),
    ("beta_uh_dry", C.c_double), ("beta_vh", C.c_double), ("beta_vh_dry", C.c_double),
    ("alpha_balance", C.c_double), ("CFL", C.c_double),
    ("evolve_max_timestep", C.c_double), ("evolve_min_timestep", C.c_double),
    ("tight_slope_limiters", C.c_int64), ("use_centroid_velocities", C.c_int64),
    ("optimise_dry_cells", C.c_int64), ("extrapolate_velocity_second_order", C.c_int64),
    ("use_sloped_mannings", C.c_int64), ("max_smallsteps", C.c_int64),
    ("default_order", C.c_int64), ("optimised_gradient_limiter", C.c_int64),
    ("use_edge_limiter", C.c_int64), ("flow_algorithm", C.c_int64),
]


class Params_t(C.Structure):
    _fields_ = PARAM_FIELDS


class State_t(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("yieldtime", C.c_double), ("finaltime", C.c_double),
        ("timestep", C.c_double), ("flux_timestep", C.c_double),
        ("recorded_max_timestep", C.c_double), ("recorded_min_timestep", C.c_double),
        ("order", C.c_int64), ("smallsteps", C.c_int64), ("number_of_steps", C.c_int64),
        ("total_steps", C.c_int64), ("stop_reason", C.c_int64), ("status", C.c_int64),
    ]


class LaunchConfig_t(C.Structure):
    _fields_ = [("flux_block", C.c_int32), ("update_block", C.c_int32),
                ("distribute_block", C.c_int32), ("steps_per_graph", C.c_int32),
                ("flux_pipelined", C.c_int32), ("dependent_launch", C.c_int32)]


class BoundaryTag_t(C.Structure):
    _fields_ = [("type", C.c_int64), ("p", C.c_double * 8)]


# every function declared in include/swgpu.h: (name, restype, argtypes)
_VP = C.c_void_p
_SIGNATURES = [
    ("swgpu_create", C.c_int, [C.POINTER(Mesh_t), C.POINTER(Params_t), C.c_int, C.POINTER(_VP)]),
    ("swgpu_create_ensemble", C.c_int, [C.POINTER(Mesh_t), _i64p, C.c_int,
                                        C.POINTER(Params_t), C.c_int, C.POINTER(_VP)]),
    ("swgpu_ensemble_size", C.c_int, [_VP, C.POINTER(C.c_int)]),
    ("swgpu_set_tracking", C.c_int, [_VP, C.c_int, C.c_double]),
    ("swgpu_get_tracking", C.c_int, [_VP, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("swgpu_get_launch_config", C.c_int, [_VP, C.POINTER(LaunchConfig_t)]),
    ("swgpu_set_launch_config", C.c_int, [_VP, C.POINTER(LaunchConfig_t)]),
    ("swgpu_ensemble_get_state", C.c_int, [_VP, C.c_int, C.POINTER(State_t)]),
    ("swgpu_ensemble_set_finaltimes", C.c_int, [_VP, _f64p]),
    ("swgpu_ensemble_mass", C.c_int, [_VP, _f64p]),
    ("swgpu_destroy", C.c_int, [_VP]),
    ("swgpu_mlp_num_params", C.c_int, []),
    ("swgpu_mlp_create", C.c_int, [_f32p, _f32p, _f32p, C.POINTER(_VP)]),
    ("swgpu_mlp_destroy", C.c_int, [_VP]),
    ("swgpu_mlp_last_error", C.c_char_p, [_VP]),
    ("swgpu_mlp_set_data", C.c_int, [_VP, _f32p, C.c_int64, _f32p, C.c_int64, _f32p]),
    ("swgpu_mlp_predict", C.c_int, [_VP, C.c_int64, C.c_int64, _VP, _f32p]),
    ("swgpu_mlp_gradients", C.c_int, [_VP, _i64p, C.c_int64, C.c_float, C.c_float,
                                       C.c_float, _f32p, _f32p, _f32p]),
    ("swgpu_mlp_train", C.c_int, [_VP, C.c_int, C.c_int64, C.c_uint64, C.c_float, C.c_float,
                                  C.c_float, C.c_float, _f32p, _f32p]),
    ("swgpu_mlp_get_params", C.c_int, [_VP, _f32p]),
    ("swgpu_last_error", C.c_char_p, [_VP]),
    ("swgpu_device_info", C.c_int, [C.c_char_p, C.c_int]),
    ("swgpu_set_quantity", C.c_int, [_VP, C.c_int, _f64p, _f64p, _f64p]),
    ("swgpu_get_quantity", C.c_int, [_VP, C.c_int, _f64p, _f64p, _f64p]),
    ("swgpu_get_boundary_values", C.c_int, [_VP, C.c_int, _f64p]),
    ("swgpu_get_explicit_update", C.c_int, [_VP, C.c_int, _f64p]),
    ("swgpu_get_semi_implicit_update", C.c_int, [_VP, C.c_int, _f64p]),
    ("swgpu_get_max_speed", C.c_int, [_VP, _f64p]),
    ("swgpu_set_boundary_tags", C.c_int, [_VP, C.POINTER(BoundaryTag_t), C.c_int]),
    ("swgpu_protect", C.c_int, [_VP]),
    ("swgpu_distribute_to_vertices_and_edges", C.c_int, [_VP]),
    ("swgpu_update_boundary", C.c_int, [_VP]),
    ("swgpu_compute_fluxes", C.c_int, [_VP, _f64p]),
    ("swgpu_compute_forcing_terms", C.c_int, [_VP]),
    ("swgpu_manning_friction_explicit", C.c_int, [_VP]),
    ("swgpu_extrapolate_second_order_sw", C.c_int, [_VP]),
    ("swgpu_balance_deep_and_shallow", C.c_int, [_VP]),
    ("swgpu_update_conserved_quantities", C.c_int, [_VP, C.c_double]),
    ("swgpu_update_other_quantities", C.c_int, [_VP]),
    ("swgpu_backup_conserved_quantities", C.c_int, [_VP]),
    ("swgpu_saxpy_conserved_quantities", C.c_int, [_VP, C.c_double, C.c_double]),
    ("swgpu_set_timestepping_method", C.c_int, [_VP, C.c_int]),
    ("swgpu_mass", C.c_int, [_VP, _f64p]),
    ("swgpu_get_state", C.c_int, [_VP, C.POINTER(State_t)]),
    ("swgpu_set_state", C.c_int, [_VP, C.POINTER(State_t)]),
    ("swgpu_evolve_start", C.c_int, [_VP, C.c_double, C.c_double, C.c_double]),
    ("swgpu_evolve_run", C.c_int, [_VP, C.c_int64, C.POINTER(State_t)]),
    ("swgpu_evolve_one_step", C.c_int, [_VP, C.POINTER(State_t)]),
    ("swgpu_evolve_run_timed", C.c_int, [_VP, C.c_int64, C.POINTER(State_t), _f64p]),
    ("swgpu_profile_steps", C.c_int, [_VP, C.c_int64, _f64p]),
    ("swgpu_synchronize", C.c_int, [_VP]),
    ("swgpu_water_volume_noalloc", C.c_int, [_VP, _VP, _VP, C.c_int64, _VP, _VP]),
]
EXPORTED_SYMBOLS = [name for name, _, _ in _SIGNATURES]

_LIB = None


class SwgpuError(RuntimeError):
    """A libswgpu call returned a nonzero status."""

    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def lib(path: str | None = None):
    """Load libswgpu.so (once).  Raises if it is absent: there is no other
    implementation to fall back to."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    # SWGPU_LIBRARY names another build of the same library (e.g. one built
    # with different launch parameters); it is still libswgpu
    p = path or os.environ.get("SWGPU_LIBRARY") or library_path()
    if not os.path.exists(p):
        raise ImportError(
            f"{p} not found: build it with anuga_cuda.build() (nvcc, sm_103a); "
            "this package has no CPU implementation")
    L = C.CDLL(p)
    for name, res, args in _SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = L
    return L


def check(status, handle=None):
    if status != 0:
        msg = lib().swgpu_last_error(handle)
        raise SwgpuError(status, msg.decode() if msg else "")


def f64p(a: np.ndarray):
    return a.ctypes.data_as(_f64p)


def i64p(a: np.ndarray):
    return a.ctypes.data_as(_i64p)
