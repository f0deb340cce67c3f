"""ctypes binding of libmsotgpu.so (include/msot_gpu.h).

The library is the only compute path: if it is missing this module raises
(there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

MSOT_OK = 0
ERRORS = {
    -1: "MSOT_EINVAL",
    -2: "MSOT_ERANGE",
    -3: "MSOT_ECUDA",
    -4: "MSOT_ENOMEM",
    -5: "MSOT_ENONFINITE",
    -6: "MSOT_ETIMEOUT",
}


class MsotError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class PlanDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("nz", C.c_int),
        ("n_det", C.c_int), ("n_t", C.c_int),
        ("radius", C.c_double),
        ("travel", C.POINTER(C.c_double)),
        ("ir_len", C.c_int),
        ("ir", C.POINTER(C.c_double)),
        ("pre_len_x", C.c_int), ("pre_len_z", C.c_int),
        ("pre_x", C.POINTER(C.c_double)),
        ("pre_z", C.POINTER(C.c_double)),
        ("norm", C.c_double),
        ("sir_len", C.c_int), ("n_sir", C.c_int),
        ("sir", C.POINTER(C.c_double)),
        ("sir_start_end", C.POINTER(C.c_int32)),
        ("sir_idx", C.POINTER(C.c_int32)),
        ("max_batch", C.c_int),
    ]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class SpmrSpec(C.Structure):
    _fields_ = [
        ("n_det", C.c_int), ("radius", C.c_double), ("coverage_deg", C.c_double),
        ("x", _dp), ("nx", C.c_int), ("z", _dp), ("nz", C.c_int),
        ("c", C.c_double), ("fs", C.c_double), ("pixel_sigma", C.c_double),
        ("elem_width", C.c_double), ("elem_height", C.c_double),
        ("elem_elev_radius", C.c_double), ("sub_x", C.c_int), ("sub_y", C.c_int),
        ("half_window", C.c_int), ("virt_x", _dp), ("virt_z", _dp),
    ]


class Tuning(C.Structure):
    _fields_ = [("fwd_wt", C.c_int), ("conv_min_blocks", C.c_int), ("tv_cluster", C.c_int),
                ("fwd_ms", C.c_double), ("transpose_ms", C.c_double), ("tv_prox_ms", C.c_double),
                ("adj_wt", C.c_int), ("fwd_staged", C.c_int)]


class SpmrInfo(C.Structure):
    _fields_ = [
        ("d_min", C.c_double), ("d_step", C.c_double), ("a_step_deg", C.c_double),
        ("n_dist", C.c_int), ("n_angle", C.c_int), ("n_sir", C.c_int), ("sir_len", C.c_int),
    ]

class ModelFields(C.Structure):
    """msot_model_fields: the reference model object's fields a plan is
    built from (MSOTmodel.m:18-48)."""
    _fields_ = [
        ("nx", C.c_int), ("nz", C.c_int), ("n_det", C.c_int), ("n_t", C.c_int),
        ("radius", C.c_double), ("travel", C.POINTER(C.c_double)),
        ("ir_hat", C.POINTER(C.c_double)), ("n_hat", C.c_int), ("eir_length", C.c_int),
        ("prefilter", C.POINTER(C.c_double)), ("sir_len", C.c_int), ("n_sir", C.c_int),
        ("sir", C.POINTER(C.c_double)), ("sir_start_end", C.POINTER(C.c_int32)),
        ("sir_idx", C.POINTER(C.c_int32)), ("norm", C.c_double), ("max_batch", C.c_int),
    ]


# name: (restype, argtypes)
SIGNATURES = {
    "msot_last_error": (C.c_char_p, []),
    "msot_version": (C.c_int, []),
    "msot_plan_create": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(_vp)]),
    "msot_plan_destroy": (C.c_int, [_vp]),
    "msot_plan_device_bytes": (C.c_size_t, [_vp]),
    "msot_forward": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_transpose": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_interp_forward": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_interp_transpose": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_interp_transpose_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_plan_set_storage": (C.c_int, [_vp, C.c_int, C.c_int]),
    "msot_estimate_norm": (C.c_int, [_vp, C.c_int, C.c_uint64, _dp, _vp]),
    "msot_rec_nn_with_L2_reg": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_double, _vp,
                                          C.c_int, _dp, _dp, _vp]),
    "msot_rec_nn_with_L2_reg_warm": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_double,
                                               _vp, _vp, C.c_int, _dp, _dp, _vp]),
    "msot_rec_nn_with_L2_reg_state": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int,
                                                C.c_double, _vp, _vp, C.c_int, _dp, _dp, _vp]),
    "msot_rec_nn_with_L1_eye_reg": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_double, _vp,
                                              C.c_int, _dp, _dp, _vp]),
    "msot_rec_nn_with_TV_reg": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_double, C.c_int,
                                          _vp, C.c_int, _dp, _dp, _vp]),
    "msot_sb_itv2": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_double, _vp]),
    "msot_itv": (C.c_int, [_vp, _dp, C.c_int, C.c_int, _vp]),
    "msot_tv_prox_path": (C.c_int, [C.c_int]),
    "msot_tune_set": (C.c_int, [C.c_char_p, C.c_int]),
    "msot_tv_prox_stats": (C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "msot_travel_times": (C.c_int, [C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp,
                                    C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    _dp]),
    "msot_spmr_query": (C.c_int, [C.POINTER(SpmrSpec), C.POINTER(SpmrInfo)]),
    "msot_spmr_tables": (C.c_int, [C.POINTER(SpmrSpec), _dp, _ip, _ip]),
    "msot_unet_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                   C.POINTER(C.c_void_p)]),
    "msot_unet_create_ch": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                      C.POINTER(C.c_void_p)]),
    "msot_unet_destroy": (C.c_int, [_vp]),
    "msot_unet_param_count": (C.c_int, [_vp, C.POINTER(C.c_size_t)]),
    "msot_unet_get_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "msot_unet_set_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "msot_unet_forward": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_unet_gradients": (C.c_int, [_vp, _vp, _vp, C.c_int, _dp, C.POINTER(C.c_float), _vp]),
    "msot_unet_adam_step": (C.c_int, [_vp, C.c_double, C.c_int, _vp]),
    "msot_unet_check": (C.c_int, [_vp]),
    "msot_travel_times_dual": (C.c_int, [C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp,
                                         C.c_int, C.c_double, C.c_double, _dp, C.c_int,
                                         C.c_double, C.c_double, C.c_double, _dp, _dp, _dp,
                                         _dp]),
    "msot_rec_nn_with_L2_reg_2": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_double,
                                            C.c_double, _vp, C.c_int, _dp, _dp, _dp, _vp]),
    "msot_laplacian_per_wavelength": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    "msot_l2_gather_probe": (C.c_int, [C.c_size_t, _dp]),
    "msot_autotune": (C.c_int, [_vp, C.c_int, _vp, C.POINTER(Tuning)]),
    "msot_prep_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_double, C.c_int, C.POINTER(_vp)]),
    "msot_prep_apply": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "msot_prep_destroy": (C.c_int, [_vp]),
    "msot_butter_response": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                       _dp]),
    "msot_dmas_cf": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, C.c_int,
                               C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               _vp, _vp, _vp, _vp, _vp]),
    "msot_backproject_waveeq": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp,
                                          C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, _dp, C.c_int, C.c_int, _vp,
                                          C.c_int, _vp, _vp]),
    "msot_launch_count": (C.c_longlong, []),
    "msot_profile_enable": (C.c_int, [C.c_int]),
    "msot_profile_kernel_name": (C.c_char_p, [C.c_int]),
    "msot_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "msot_plan_valid": (C.c_int, [_vp]),
    "msot_plan_create_from_model": (C.c_int, [C.POINTER(ModelFields), C.POINTER(_vp)]),
    "msot_plan_norm": (C.c_double, [_vp]),
    "msot_plan_shape": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "msot_host_apply": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _dp]),
    "msot_host_rec_nn_with_L2_reg": (C.c_int, [_vp, _dp, C.c_int, C.c_int, C.c_double,
                                               C.c_double, _dp, _dp, _dp, _dp]),
    "msot_host_rec_nn_with_L1_eye_reg": (C.c_int, [_vp, _dp, C.c_int, C.c_int, C.c_double,
                                                   _dp, _dp, _dp]),
    "msot_host_rec_nn_with_TV_reg": (C.c_int, [_vp, _dp, C.c_int, C.c_int, C.c_double, _dp,
                                               _dp, _dp]),
    "msot_mex_forwardDelayAndSum": (C.c_int, [_dp, C.c_int, C.c_int, _dp, C.c_int, C.c_int,
                                              C.c_double, _dp]),
    "msot_mex_transposeDelayAndSum": (C.c_int, [_dp, C.c_int, C.c_int, C.c_int, _dp, C.c_int,
                                                C.c_double, _dp]),
    "msot_mex_forward": (C.c_int, [_dp, C.c_int, C.c_int, _ip, _dp, C.c_int, _dp, C.c_int,
                                   C.c_int, C.c_int, _ip, C.c_double, _dp]),
    "msot_mex_transpose": (C.c_int, [_dp, C.c_int, C.c_int, C.c_int, _ip, _dp, C.c_int, _dp,
                                     C.c_int, C.c_int, _ip, C.c_double, _dp]),
}

_LIB = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Load the CUDA library (optionally building it first)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(
                f"{path} is missing: build it with __graft_entry__.build() or "
                "python mb-rec-msot_gb300/msot_gb300/_build.py (no CPU fallback exists)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def check(rc: int) -> None:
    if rc != MSOT_OK:
        msg = load().msot_last_error()
        raise MsotError(rc, msg.decode() if msg else "")
