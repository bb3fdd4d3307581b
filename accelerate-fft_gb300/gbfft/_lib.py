"""ctypes binding of libgbfft.so (the C ABI declared in include/gbfft.h).

The library is the product path: if it is missing or fails to load, every
call raises -- there is no CPU or library fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbfft.so")

OK = 0
ERR_INVALID_ARG = 1
ERR_UNSUPPORTED = 2
ERR_ALLOC = 3
ERR_CUDA = 4
ERR_NULL_PLAN = 5
ERR_TIMEOUT = 6
ERR_INTERNAL = 7
ERR_TOO_LARGE = 8

FORWARD, REVERSE, INVERSE = -1, 1, 2
C32, C64 = 0, 1
KIND_MANY, KIND_FULL = 0, 1
PLAIN, SPLIT_FP16 = 0, 1
OPT_SHIFT_OUT, OPT_ISHIFT_OUT, OPT_CENTRE_IN = 1, 2, 4

_vp = ctypes.c_void_p
_i64p = ctypes.POINTER(ctypes.c_int64)
_i = ctypes.c_int
_i64 = ctypes.c_int64
_sz = ctypes.c_size_t

# name -> (restype, argtypes); every function declared in include/gbfft.h
SIGNATURES = {
    "gbfft_error_string": (ctypes.c_char_p, [_i]),
    "gbfft_version": (_i, []),
    "gbfft_plan_create": (_i, [ctypes.POINTER(_vp), _i, _i64p, _i, _i, _i]),
    "gbfft_plan_destroy": (_i, [_vp]),
    "gbfft_exec": (_i, [_vp, _i, _vp, _vp, _vp]),
    "gbfft_exec_ex": (_i, [_vp, _i, _vp, _vp, _vp, _i]),
    "gbfft_probe_tile_copy": (_i, [_i64, _i64, _i, _vp, _vp, _vp]),
    "gbfft_plan_get": (_i, [ctypes.POINTER(_vp), _i, _i64p, _i, _i, _i]),
    "gbfft_fft": (_i, [_i, _i, _i64p, _i, _i, _vp, _vp, _vp]),
    "gbfft_cache_clear": (_i, []),
    "gbfft_exec_range": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp]),
    "gbfft_exec_status": (_i, [_vp, _vp]),
    "gbfft_plan_info": (_i, [_vp, ctypes.POINTER(_sz), ctypes.POINTER(_i)]),
    "gbfft_plan_describe": (_i, [_vp, ctypes.c_char_p, _sz]),
    "gbfft_plan_pass_kernel": (_i, [_vp, _i, ctypes.c_char_p, _sz]),
    "gbfft_autotune": (_i, [_i, _i64p, _i, _i, _i, _vp, ctypes.c_char_p, _sz]),
    "gbfft_dftG": (_i, [_i, _i64p, _i, _vp, _vp, _vp, _vp]),
    "gbfft_dftGS": (_i, [_i, _i64p, _i, _i64, _vp, _vp, _vp, _vp]),
    "gbfft_centre": (_i, [_i, _i64p, _i, _vp, _vp, _vp]),
    "gbfft_shift": (_i, [_i, _i64p, _i, _i, _vp, _vp, _vp]),
    "gbfft_tune_load": (_i, [ctypes.c_char_p]),
    "gbfft_tune_clear": (_i, []),
    "gbfft_tune_count": (_i, []),
    "gbfft_plan_explain": (_i, [_i, _i64p, _i, _i, _i, ctypes.c_char_p, _sz]),
    "gbfft_ragged_plan_create": (_i, [ctypes.POINTER(_vp), _i64, _i64p, _i64p,
                                      ctypes.POINTER(_i), _i]),
    "gbfft_ragged_autotune": (_i, [_i64, _i64p, _i64p, ctypes.POINTER(_i), _i, _vp, ctypes.c_char_p, _sz]),
    "gbfft_ragged_exec": (_i, [_vp, _vp, _vp, _vp]),
    "gbfft_ragged_exec_per_transform": (_i, [_vp, _vp, _vp, _vp]),
    "gbfft_ragged_plan_destroy": (_i, [_vp]),
    "gbfft_ragged_status": (_i, [_vp, _vp]),
    "gbfft_specconv_plan_create": (_i, [ctypes.POINTER(_vp), _i64, _i64, _i64, _i64, _i]),
    "gbfft_specconv_fwd": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "gbfft_specconv_bwd": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbfft_specconv_plan_destroy": (_i, [_vp]),
    "gbfft_fft_noalloc": (_i, [_i, _i64, _i64, _i, _vp, _vp, _vp]),
}

_lib = None


class GbfftError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = error_string(status) if _lib is not None else "status %d" % status
        super().__init__("%s: %s (status %d)" % (what or "gbfft", msg, status))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GbfftError(ERR_INTERNAL, "libgbfft.so not built (run accelerate-fft_gb300/build.py)")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def error_string(status):
    return lib().gbfft_error_string(int(status)).decode()


def check(status, what=""):
    if status != OK:
        raise GbfftError(status, what)
