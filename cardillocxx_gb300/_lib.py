"""ctypes binding of libcdx.so (the C ABI in include/cdx.h).

The library must be built in-tree (cardillocxx_gb300/libcdx.so, see build.py). Loading fails
loudly when it is missing: there is no Python or CPU fallback for any engine call.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcdx.so")

_P = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int32)

CDX_OK = 0
STATUS = {0: "CDX_OK", 1: "CDX_ERR_ARG", 2: "CDX_ERR_CUDA", 3: "CDX_ERR_OVERFLOW", 4: "CDX_ERR_NONFINITE",
          5: "CDX_ERR_TIMEOUT", 6: "CDX_ERR_UNSUPPORTED", 7: "CDX_ERR_STATE"}
PRECISION_FP64 = 0
PRECISION_SPLIT = 1


class CdxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class CdxConfig(C.Structure):
    _fields_ = [
        ("sim_dt", C.c_double),
        ("sim_T", C.c_double),
        ("sim_gravity", C.c_double * 3),
        ("moreau_theta", C.c_double),
        ("moreau_implicit_gyroscopy", C.c_int32),
        ("friction_enable", C.c_int32),
        ("friction_combine", C.c_int32),
        ("friction_default_mu", C.c_double),
        ("restitution_default_normal", C.c_double),
        ("restitution_default_tangential", C.c_double),
        ("pj_max_iterations", C.c_int32),
        ("pj_warmstart", C.c_int32),
        ("pj_tol_abs", C.c_double),
        ("pj_tol_rel", C.c_double),
        ("pj_alpha", C.c_double),
        ("pj_relaxation", C.c_double),
        ("solver_type", C.c_int32),
        ("collision_security_margin", C.c_double),
        ("collision_match_max_dist", C.c_double),
        ("collision_broadphase", C.c_int32),
        ("gpu_precision", C.c_int32),
        ("gpu_residual_tol", C.c_double),
        ("gpu_check_every", C.c_int32),
        ("gpu_block", C.c_int32),
        ("gpu_contact_capacity_factor", C.c_double),
        ("gpu_use_graph", C.c_int32),
        ("gpu_autotune", C.c_int32),
        ("gpu_sweep_variant", C.c_int32),
        ("gpu_sync_counts", C.c_int32),
        ("pj_nesterov", C.c_int32),
        ("pj_nesterov_beta_threshold", C.c_double),
        ("pj_nesterov_restart_limit", C.c_int32),
        ("pj_chebyshev", C.c_int32),
        ("pj_anderson", C.c_int32),
        ("pj_anderson_m", C.c_int32),
        ("pj_rdiag_true_delassus", C.c_int32),
        ("output_interval_steps", C.c_int32),
        ("output_write_contact_manifolds", C.c_int32),
        ("output_folder", C.c_char * 256),
        ("output_filename_prefix", C.c_char * 128),
        ("gpu_coop_smem_contacts", C.c_int32),
        ("gpu_coop_blocks", C.c_int32),
        ("gpu_tune_alpha", C.c_int32),
        ("gpu_coop_wait_ns", C.c_int64),
        ("condensed_sweep_mode", C.c_int32),
        ("gpu_tune_alpha_every", C.c_int32),
    ]


class CdxScene(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_int32),
        ("pos", _P), ("quat", _P), ("vel", _P), ("omega", _P),
        ("radius", _P), ("mass", _P), ("inertia", _P), ("mu", _P), ("rest_n", _P), ("rest_t", _P),
        ("body_scene", _PI),
        ("num_statics", C.c_int32),
        ("static_kind", _PI),
        ("static_pos", _P), ("static_quat", _P), ("static_vel", _P), ("static_omega", _P),
        ("static_dir", _P), ("static_radius", _P),
        ("static_mu", _P), ("static_rest_n", _P), ("static_rest_t", _P),
        ("static_scene", _PI),
        ("num_scenes", C.c_int32),
        ("static_half_length", _P),
        ("static_half_extents", _P),
    ]


class CdxStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("num_contacts", C.c_int32),
        ("num_rows", C.c_int32),
        ("iterations", C.c_int32),
        ("reallocations", C.c_int32),
        ("residual", C.c_double),
        ("residual_last", C.c_double),
        ("ms_collision", C.c_double),
        ("ms_setup", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_integrate", C.c_double),
        ("solve_bytes_per_iter", C.c_double),
        ("kernel_launches", C.c_int64),
        ("contact_variant", C.c_int32),
        ("autotune_runs", C.c_int32),
        ("redone_steps", C.c_int32),
        ("graph_steps", C.c_int64),
        ("sweep_variant", C.c_int32),
        ("levels", C.c_int32),
    ]


class CdxGenParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("num_scenes", C.c_int32),
        ("num_bodies", C.c_int32),
        ("nb_lo", C.c_int32),
        ("nb_hi", C.c_int32),
        ("r_lo", C.c_double),
        ("r_hi", C.c_double),
        ("density", C.c_double),
        ("box", C.c_double * 3),
        ("mu", C.c_double),
        ("mu_lo", C.c_double),
        ("mu_hi", C.c_double),
        ("v_sigma", C.c_double),
        ("drum_radius", C.c_double),
        ("drum_length", C.c_double),
        ("drum_omega", C.c_double),
        ("seed", C.c_uint64),
        ("max_attempts", C.c_int32),
    ]


# every exported symbol declared in include/cdx.h: (name, restype, argtypes)
SIGNATURES = [
    ("cdx_config_default", C.c_int, [C.POINTER(CdxConfig)]),
    ("cdx_config_set", C.c_int, [C.POINTER(CdxConfig), C.c_char_p, C.c_char_p]),
    ("cdx_config_from_file", C.c_int, [C.c_char_p, C.POINTER(CdxConfig)]),
    ("cdx_create", C.c_int, [C.POINTER(CdxConfig), C.POINTER(C.c_void_p)]),
    ("cdx_destroy", None, [C.c_void_p]),
    ("cdx_last_error", C.c_char_p, [C.c_void_p]),
    ("cdx_load_scene", C.c_int, [C.c_void_p, C.POINTER(CdxScene)]),
    ("cdx_step", C.c_int, [C.c_void_p, C.c_int32]),
    ("cdx_synchronize", C.c_int, [C.c_void_p]),
    ("cdx_get_state", C.c_int, [C.c_void_p, _P, _P, _P, _P]),
    ("cdx_set_state", C.c_int, [C.c_void_p, _P, _P, _P, _P]),
    ("cdx_get_stats", C.c_int, [C.c_void_p, C.POINTER(CdxStats)]),
    ("cdx_get_contacts", C.c_int, [C.c_void_p, _PI, _PI, _P, _P, _P, _PI]),
    ("cdx_set_contacts", C.c_int, [C.c_void_p, C.c_int32, _PI, _PI, _P, _P]),
    ("cdx_set_config", C.c_int, [C.c_void_p, C.POINTER(CdxConfig)]),
    ("cdx_get_scene_solve", C.c_int, [C.c_void_p, C.POINTER(C.c_float), _PI, C.c_int32]),
    ("cdx_set_static_motion", C.c_int, [C.c_void_p, C.c_int32, _PI, _P, _P, _P, _P]),
    ("cdx_get_static_state", C.c_int, [C.c_void_p, _P, _P, _P, _P]),
    ("cdx_track", C.c_int, [C.c_void_p, C.c_int32, C.c_char_p]),
    ("cdx_output_flush", C.c_int, [C.c_void_p]),
    ("cdx_set_trace", C.c_int, [C.c_void_p, C.c_int32]),
    ("cdx_get_trace", C.c_int, [C.c_void_p, _P, C.c_int64, C.POINTER(C.c_int64)]),
    ("cdx_set_timing", C.c_int, [C.c_void_p, C.c_int32]),
    ("cdx_stream", C.c_void_p, [C.c_void_p]),
    ("cdx_time_sweeps", C.c_int, [C.c_void_p, C.c_int32, _P, _P, _P, _P]),
    ("cdx_selftest_nr64", C.c_int, [C.c_void_p, C.c_int32, _P, _P, _P]),
    ("cdx_adj_create", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    ("cdx_adj_destroy", None, [C.c_void_p]),
    ("cdx_adj_last_error", C.c_char_p, [C.c_void_p]),
    ("cdx_adj_forward", C.c_int, [C.c_void_p, C.c_int32, _P, _P, _P, _P, _P, _P, _P]),
    ("cdx_adj_backward", C.c_int, [C.c_void_p, _P, _P, _P, _P, _P, _P, _P]),
    ("cdx_adj_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    ("cdx_adj_contact_counts", C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    ("cdx_split_variant_count", C.c_int32, []),
    ("cdx_split_variant_name", C.c_char_p, [C.c_int32]),
    ("cdx_pj_solve_csr", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _PI, _PI, _P, _P, _P, _P, _P, _P,
                                   _P, _P, _P, C.c_double, C.c_double, C.c_int32, C.c_double, C.c_double, _P, _P,
                                   _PI]),
    ("cdx_pj_solve_csr_cfg", C.c_int, [C.c_void_p, C.POINTER(CdxConfig), C.c_int32, C.c_int32, C.c_int32, _PI, _PI,
                                       _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_double, _P, _P, _PI]),
    ("cdx_pj_solve_csr_noalloc", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _PI, _PI, _P, _P, _P, _P,
                                           _P, _P, _P, _P, _P, C.c_double, C.c_double, C.c_int32, C.c_double,
                                           C.c_double, _P, _P, _PI, C.c_char_p, C.c_int32]),
    ("cdx_gen_create", C.c_int, [C.POINTER(CdxGenParams), C.POINTER(C.c_void_p)]),
    ("cdx_gen_view", C.c_int, [C.c_void_p, C.POINTER(CdxScene)]),
    ("cdx_gen_destroy", None, [C.c_void_p]),
]

_lock = threading.Lock()
_lib = None


def lib():
    """Load libcdx.so (raises when it is not built; never falls back)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"libcdx.so is not built at {LIB_PATH}; run cardillocxx_gb300/build.py")
            L = C.CDLL(LIB_PATH)
            for name, res, args in SIGNATURES:
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def dp(a):
    return a.ctypes.data_as(_P) if a is not None else None


def ip(a):
    return a.ctypes.data_as(_PI) if a is not None else None
