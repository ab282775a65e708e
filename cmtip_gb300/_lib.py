"""ctypes binding of ``libcmtip_gb300.so`` (the C ABI declared in include/cmtip_gb300.h).

The library is built in-tree by ``cmtip_gb300.build``; there is no other implementation
of these operations in the package, so a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcmtip_gb300.so")

CMT_OK = 0
CMT_ERR_ARG = 1
CMT_ERR_RANGE = 2
CMT_ERR_OOM = 3
CMT_ERR_CUDA = 4
CMT_ERR_TIMEOUT = 5
CMT_ERR_CUFFT = 6
CMT_ERR_STATE = 7

CMT_REAL_IN = 1
CMT_REAL_OUT = 2
CMT_MODEORD_FFT = 4

_vp = ctypes.c_void_p
_i32 = ctypes.c_int
_i64 = ctypes.c_int64
_f64 = ctypes.c_double

# name -> argtypes (restype int unless listed in _RESTYPE)
SIGNATURES = {
    "cmt_plan_create": [_i32, _i32, _i32, _f64, _i32, _f64, _vp, ctypes.POINTER(_vp)],
    "cmt_plan_create_derived": [_vp, _i32, _i32, _i32, ctypes.POINTER(_vp)],
    "cmt_plan_info": [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_f64),
                      ctypes.POINTER(_i32), ctypes.POINTER(_i64)],
    "cmt_set_pts": [_vp, _i64, _vp, _vp, _vp],
    "cmt_set_pts_quat": [_vp, _i64, _vp, _i64, _vp, _f64],
    "cmt_execute": [_vp, _vp, _vp, _vp, _f64, _i32],
    "cmt_execute_pair": [_vp, _vp, _vp, _vp, _f64],
    "cmt_plan_destroy": [_vp],
    "cmt_plan_set_stream": [_vp, _vp],
    "cmt_plan_profile": [_vp, _i32],
    "cmt_plan_profile_read": [_vp, _vp, _vp, _i32, ctypes.POINTER(_i32)],
    "cmt_plan_prepare_pair": [_vp],
    "cmt_plan_set_tuning": [_vp, _i32, _i32],
    "cmt_plan_get_tuning": [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
    "cmt_batch_create": [_i32, _vp, _vp, ctypes.POINTER(_vp)],
    "cmt_batch_execute": [_vp, _vp, _vp, _vp, _vp, _i32],
    "cmt_batch_profile": [_vp, _i32],
    "cmt_batch_last_ms": [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(_i64)],
    "cmt_batch_destroy": [_vp],
    "cmt_bin_clip": [_i32, _vp, _i64, _i32, _i32, _i32, _i32, _vp, _i64, _vp, _vp],
    "cmt_inverse_rotations": [_vp, _i64, _vp, _vp],
    "cmt_cg_create": [_i32, _i32, _i32, _vp, ctypes.POINTER(_vp)],
    "cmt_cg_set_kernel": [_vp, _vp],
    "cmt_cg_set_operator": [_vp, _vp, _vp, _f64, _f64, _f64],
    "cmt_cg_set_pair_plan": [_vp, _vp],
    "cmt_cg_matvec": [_vp, _vp, _vp],
    "cmt_cg_solve": [_vp, _vp, _vp, _i32, _f64, _f64, _i32, ctypes.POINTER(_i32), ctypes.POINTER(_f64)],
    "cmt_cg_solve_many": [_i32, _vp, _vp, _vp, _i32, _f64, _f64, _vp, _vp],
    "cmt_cg_destroy": [_vp],
    "cmt_support_from_estimate": [_vp, _i32, _vp, _vp, _i32, _vp],
    "cmt_support_from_estimate_noalloc": [_vp, _i32, _vp, _i32, _vp],
    "cmt_phase_create": [_i32, _i32, _vp, ctypes.POINTER(_vp)],
    "cmt_phase_set_stream": [_vp, _vp],
    "cmt_phase_amplitudes": [_vp, _vp, _vp, _i32, _vp, _vp],
    "cmt_phase_create_support": [_vp, _vp, _i32, _vp],
    "cmt_phase_step": [_vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cmt_phase_er": [_vp, _vp, _vp, _vp, _vp, _f64, _i32],
    "cmt_phase_hio": [_vp, _f64, _vp, _vp, _vp, _vp, _f64, _i32],
    "cmt_phase_shrink_wrap": [_vp, _f64, _vp, _i32, _vp, _vp],
    "cmt_phase_center_of_mass": [_vp, _vp, _vp, _vp],
    "cmt_phase_roll": [_vp, _vp, _vp, _i32, _i32, _i32],
    "cmt_phase_autocorrelation": [_vp, _vp, _vp],
    "cmt_phase_destroy": [_vp],
    "cmt_match_create": [_i64, _i32, _vp, ctypes.POINTER(_vp)],
    "cmt_match_set_data": [_vp, _i64, _vp, _vp],
    "cmt_match_set_refs": [_vp, _i64, _vp, _i32],
    "cmt_match_run": [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_i32)],
    "cmt_match_run_many": [_i32, _vp, _vp, _vp, _vp, _vp, _vp],
    "cmt_match_profile": [_vp, _i32],
    "cmt_match_set_wait_limit": [_vp, _f64],
    "cmt_match_set_tile": [_vp, _i32, _i32],
    "cmt_match_stall_loads": [_vp, _i32],
    "cmt_match_last_ms": [_vp, ctypes.POINTER(ctypes.c_float)],
    "cmt_match_stats": [_vp, ctypes.POINTER(_f64)],
    "cmt_match_destroy": [_vp],
    "cmt_last_error": [],
    "cmt_version": [],
}
_RESTYPE = {"cmt_last_error": ctypes.c_char_p, "cmt_version": ctypes.c_char_p}

_lib = None
_lock = threading.Lock()


class CmtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cmtip_gb300 error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise ImportError(f"{path} not found: build it with `python -m cmtip_gb300.build` "
                                  "(there is no non-CUDA implementation)")
            lib = ctypes.CDLL(path)
            for name, args in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = _RESTYPE.get(name, ctypes.c_int)
            _lib = lib
    return _lib


def check(code: int):
    if code == CMT_OK:
        return
    msg = load().cmt_last_error().decode(errors="replace")
    if code == CMT_ERR_RANGE:
        # the reference asserts |x| < 3 pi (cmtip/nufft/forward.py:27, adjoint.py:29)
        raise AssertionError(msg)
    if code == CMT_ERR_ARG:
        raise ValueError(msg)
    if code == CMT_ERR_OOM:
        raise MemoryError(msg)
    raise CmtError(code, msg)


def call(name: str, *args):
    check(getattr(load(), name)(*args))


def version() -> str:
    return load().cmt_version().decode()
