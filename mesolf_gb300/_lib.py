"""ctypes bindings of libmesolf_lf.so (the C ABI in include/mesolf_lf.h)."""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmesolf_lf.so")

MLF_OK = 0
MLF_ERR_INVALID = 1
MLF_ERR_CUDA = 2
MLF_ERR_NOMEM = 3
MLF_ERR_UNSUPPORTED = 4
MLF_ERR_TIMEOUT = 5
MLF_ERR_CANCELLED = 6

MLF_PREC_FP32 = 0
MLF_PREC_BF16X3 = 1
MLF_PREC_BF16 = 2
MLF_PREC_BF16X2 = 3
MLF_PREC_FP16 = 4
MLF_PREC_FP16X2 = 5
MLF_PREC_FP16X3 = 6
MLF_DETREND_PIXELWISE = 0
MLF_DETREND_GLOBAL = 1
MLF_DTYPE_F32 = 0
MLF_DTYPE_U16 = 1

#: Every symbol declared in include/mesolf_lf.h, with (restype, argtypes).
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
SIGNATURES = {
    "mlf_version": (ctypes.c_int, []),
    "mlf_probe_fp32_peak": (ctypes.c_int, [ctypes.c_double, ctypes.POINTER(ctypes.c_double), _vp]),
    "mlf_probe_wait_timeout": (ctypes.c_int, [ctypes.c_uint32, _vp]),
    "mlf_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "mlf_conv_vec": (ctypes.c_int, [_vp, _i64, _i64, _i64, _vp, _i64, _i32, _vp, _vp]),
    "mlf_conv_vec_ex": (ctypes.c_int, [_vp, _i64, _i64, _i64, _vp, _i64, _i32, _vp, _i32, _vp]),
    "mlf_conv_vec_accumulate": (ctypes.c_int, [_vp, _i64, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _i32, _i64,
                                               _vp, _vp]),
    "mlf_psf_create": (ctypes.c_int, [_vp, _vp, _i64, _i32, _i64, ctypes.POINTER(_vp), _vp]),
    "mlf_psf_destroy": (ctypes.c_int, [_vp]),
    "mlf_psf_info": (ctypes.c_int, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "mlf_psf_weights": (ctypes.c_int, [_vp, _vp]),
    "mlf_psf_device_bytes": (_i64, [_vp]),
    "mlf_solver_create": (ctypes.c_int, [_vp, _i64, _i64, ctypes.POINTER(_vp)]),
    "mlf_solver_destroy": (ctypes.c_int, [_vp]),
    "mlf_solver_device_bytes": (_i64, [_vp]),
    "mlf_solver_run": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp]),
    "mlf_rl_solve": (ctypes.c_int, [_vp, _i64, _i64, _vp, _vp, _i64, _i32, _i64, _i32, _i32, _vp, _vp, _vp]),
    "mlf_forward_view": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "mlf_backward_view": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "mlf_rl_view_step": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, ctypes.c_double, _vp]),
    "mlf_sample_filter": (ctypes.c_int, [_vp, _vp, _vp]),
    "mlf_rl_view_step_prec": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, ctypes.c_double, _i32, _vp]),
    "mlf_forward_view_prec": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i32, _vp, _vp]),
    "mlf_forward_view_static": (ctypes.c_int, [_vp, _vp, _i64, _i64, _i32, _i32, _vp, _vp]),
    "mlf_batch_create": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "mlf_batch_destroy": (ctypes.c_int, [_vp]),
    "mlf_batch_device_bytes": (_i64, [_vp]),
    "mlf_batch_run": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp]),
    "mlf_batch_cancel": (ctypes.c_int, [_vp]),
    "mlf_batch_cancelled": (ctypes.c_int, [_vp]),
    "mlf_solver_cancel": (ctypes.c_int, [_vp]),
    "mlf_solver_cancelled": (ctypes.c_int, [_vp]),
    "mlf_solver_create_variant": (ctypes.c_int, [_vp, _i64, _i64, _i32, _vp]),
    "mlf_solver_run_peeling": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mlf_batch_plan_bytes": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, ctypes.POINTER(_i64)]),
    "mlf_forward_project": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp]),
    "mlf_batch_forward_project": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp]),
    "mlf_rectify_frames": (ctypes.c_int, [_vp, _i32, _i64, _i64, _i64, _vp, ctypes.c_double, ctypes.c_double, _i32,
                                          ctypes.c_double, _i64, _i64, _i64, _i64, _i64, _i32, _i32, _vp,
                                          ctypes.POINTER(_i64), _vp]),
    "mlf_summary_image": (ctypes.c_int, [_vp, _i64, _i64, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _vp]),
    "mlf_summary_image_ex": (ctypes.c_int, [_vp, _i64, _i64, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _vp,
                                            _vp]),
}


class MLFStats(ctypes.Structure):
    _fields_ = [("n_views", ctypes.c_int32), ("iterations", ctypes.c_int32), ("gpu_ms", ctypes.c_double),
                ("view_ms", ctypes.c_double), ("view_kernel_ms", ctypes.c_double),
                ("view_kernel_launches", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("fwd_splits", ctypes.c_int32), ("fwd_stages", ctypes.c_int32), ("bwd_xbufs", ctypes.c_int32),
                ("tuned", ctypes.c_int32), ("rel_change", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MesoLFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[mlf status {code}] {msg}")
        self.code = code


_lib = None


def load(path: str | None = None):
    """Load (once) and return the shared library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libmesolf_lf.so not built at {p}; run mesolf_gb300.build.build()")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != MLF_OK:
        buf = ctypes.create_string_buffer(1024)
        code = load().mlf_last_error(buf, len(buf))
        raise MesoLFError(status, buf.value.decode(errors="replace") or f"code {code}")
    return status
