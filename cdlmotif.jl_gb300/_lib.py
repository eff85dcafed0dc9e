"""ctypes binding of libcdlgb.so (the C ABI declared in include/cdlgb.h).

The library is built in-tree (``build.py``) and loaded from ``lib/libcdlgb.so``;
there is no fallback: if it is missing, importing the package's compute functions
raises."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcdlgb.so")

STATUS = {0: "OK", -1: "EINVAL", -2: "ENOMEM_BUDGET", -3: "ECUDA", -4: "ETIMEOUT",
          -5: "ESTATE", -6: "ENOTSUP"}


class CdlgbParams(C.Structure):
    _fields_ = [
        ("M", C.c_int32), ("filter_size", C.c_int32),
        ("rho", C.c_float), ("sigma", C.c_float), ("lambda_", C.c_float),
        ("csc_iter_num", C.c_int32), ("cdl_iter_num", C.c_int32), ("iter_num", C.c_int32),
        ("std_threshold_multiplier", C.c_float),
        ("sherman_const_csc", C.c_float), ("sherman_const_cdl", C.c_float),
        ("device", C.c_int32), ("init_mode", C.c_int32), ("fft_mode", C.c_int32),
        ("hbm_budget_bytes", C.c_uint64),
        ("stop_tol", C.c_float), ("track_residuals", C.c_int32),
    ]


# every exported symbol with its ctypes signature (restype, argtypes)
_vp = C.c_void_p
_i32p = C.POINTER(C.c_int32)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)
SIGNATURES = {
    "cdlgb_params_default": (C.c_int, [C.POINTER(CdlgbParams)]),
    "cdlgb_create": (C.c_int, [C.POINTER(CdlgbParams), C.POINTER(_vp)]),
    "cdlgb_destroy": (C.c_int, [_vp]),
    "cdlgb_last_error": (C.c_char_p, [_vp]),
    "cdlgb_footprint": (C.c_int, [C.POINTER(CdlgbParams), C.c_int32, C.c_int32, C.POINTER(C.c_uint64)]),
    "cdlgb_load_data": (C.c_int, [_vp, _f32p, C.c_int32, C.c_int32]),
    "cdlgb_load_fasta": (C.c_int, [_vp, C.c_char_p, C.c_size_t, C.c_int32, _i32p, _i32p, _i32p]),
    "cdlgb_dims": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p, _i32p]),
    "cdlgb_init_state": (C.c_int, [_vp, _f32p, _f32p, C.c_uint64]),
    "cdlgb_code_update": (C.c_int, [_vp, C.c_int32]),
    "cdlgb_dict_update": (C.c_int, [_vp, C.c_int32]),
    "cdlgb_objective": (C.c_int, [_vp, _f64p]),
    "cdlgb_update_best": (C.c_int, [_vp, _f64p, _i32p]),
    "cdlgb_run_outer": (C.c_int, [_vp, C.c_int32, _f64p]),
    "cdlgb_code_threshold": (C.c_int, [_vp, _f64p]),
    "cdlgb_get": (C.c_int, [_vp, C.c_int32, _vp, C.c_size_t]),
    "cdlgb_scan_fwd": (C.c_int, [_vp, _f32p, _i32p, _f32p, C.c_int32, C.c_int32, _i32p]),
    "cdlgb_scan_both": (C.c_int, [_vp, _f32p, _i32p, _f32p, C.c_int32, C.c_int32, _i32p, _f32p, _u8p]),
    "cdlgb_select_nonoverlapping": (C.c_int, [_vp, _i32p, _f32p, _u8p, _i32p, C.c_int32]),
    "cdlgb_pvalue_thresholds": (C.c_int, [_vp, _f32p, _i32p, C.c_int32, C.c_int32, C.c_double, _f32p]),
    "cdlgb_autotune": (C.c_int, [_vp, C.c_int32, C.POINTER(C.c_double), _i32p, _i32p, _i32p, _i32p, _i32p]),
    "cdlgb_count_pfms": (C.c_int, [_vp, _i32p, _u8p, _i32p, C.c_int32, C.c_int32, _i32p, _i32p]),
    "cdlgb_counts_to_pfms": (C.c_int, [_i32p, _i32p, _i32p, C.c_int32, C.c_int32, C.c_float,
                                       C.c_float, C.c_int32, C.c_int32, _f32p]),
    "cdlgb_extend_positions": (C.c_int, [_vp, _i32p, _u8p, _i32p, C.c_int32, _f32p, C.c_float,
                                         C.c_float, C.c_float, _i32p, _i32p]),
    "cdlgb_rescore_positions": (C.c_int, [_vp, _f32p, _i32p, _i32p, C.c_int32, C.c_int32, _f32p]),
    "cdlgb_trim_pfms": (C.c_int, [_f32p, _i32p, C.c_int32, C.c_int32, _f32p, _i32p, _f32p,
                                  C.c_int32, _i32p, _i32p]),
    "cdlgb_make_background": (C.c_int, [_vp, C.c_int32, C.c_uint64]),
    "cdlgb_select_data": (C.c_int, [_vp, C.c_int32]),
    "cdlgb_fisher_evalues": (C.c_int, [_i32p, _i32p, C.c_int32, C.c_int32, _f64p]),
    "cdlgb_transfac_format": (C.c_int64, [_f32p, C.c_int32, C.c_int32, C.c_char_p, C.c_size_t]),
    "cdlgb_set_stream": (C.c_int, [_vp, _vp]),
    "cdlgb_profile": (C.c_int, [_vp, C.c_int32]),
    "cdlgb_profile_read": (C.c_int, [_vp, _f64p, _i64p, _i64p, _i64p, C.c_int32]),
    "cdlgb_ar_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(_vp)]),
    "cdlgb_ar_destroy": (C.c_int, [_vp]),
    "cdlgb_ar_last_error": (C.c_char_p, [_vp]),
    "cdlgb_ar_record": (C.c_int, [_vp, _vp, C.c_double, C.c_int32, C.c_int32, _i32p]),
    "cdlgb_ar_info": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p, C.c_int32]),
    "cdlgb_ar_topology": (C.c_int, [_vp, _i32p, _i32p, _i32p]),
    "cdlgb_ar_pair_pfms": (C.c_int, [_vp, _vp, _i32p, C.c_int32, C.c_int32, _f32p, _i32p]),
    "cdlgb_objective_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32,
                                          C.c_int32, C.c_float, _f64p, _vp]),
}

class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int32), ("device", C.c_int32), ("iter_num", C.c_int32),
                ("keep_codes", C.c_int32), ("pad_friendly", C.c_int32),
                ("hbm_budget_bytes", C.c_uint64), ("seed", C.c_uint64)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("N", C.c_int32), ("L4", C.c_int32),
                ("M", C.c_int32), ("Lg", C.c_int32), ("outer_done", C.c_int32),
                ("footprint_bytes", C.c_uint64), ("obj_best", C.c_double),
                ("code_thresh", C.c_double), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("t_now", C.c_double), ("error", C.c_char * 256)]


SIGNATURES.update({
    "cdlgb_server_create": (C.c_int, [C.POINTER(CdlgbParams), C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "cdlgb_server_submit": (C.c_int, [_vp, _f32p, C.c_int32, C.c_int32, _i64p]),
    "cdlgb_server_submit_fasta": (C.c_int, [_vp, C.c_char_p, C.c_size_t, C.c_int32, _i64p]),
    "cdlgb_server_poll": (C.c_int, [_vp, C.c_int64, C.c_int32, C.POINTER(RequestInfo)]),
    "cdlgb_server_fetch": (C.c_int, [_vp, C.c_int64, _f32p, C.c_size_t, _f64p, C.c_int32, _f32p,
                                     C.c_size_t]),
    "cdlgb_server_release": (C.c_int, [_vp, C.c_int64]),
    "cdlgb_server_stats": (C.c_int, [_vp, _i32p, _i32p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "cdlgb_server_last_error": (C.c_char_p, [_vp]),
    "cdlgb_server_destroy": (C.c_int, [_vp]),
})

_lib = None


def lib() -> C.CDLL:
    """Load libcdlgb.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libcdlgb.so is not built ({LIB_PATH}); run buildlib.py (or __graft_entry__.build()) first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a, ctype):
    """ctypes pointer to a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))
