"""ctypes binding of libqzgpu.so (the C ABI declared in include/qzgpu.h).

The library is built in-tree by ``qz_gb300.build``.  There is no CPU fallback:
if the library is missing or no GPU is usable, calls raise ``QzGpuError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

QZGPU_NO_ERROR = 0
QZGPU_BAD_PARAMETER = -1
QZGPU_NOT_ENOUGH_MEMORY = -2
QZGPU_NOT_COMPRESSIBLE = -3
QZGPU_NOT_SUPPORTED = -4
QZGPU_UNEXPECTED_EOB = -5
QZGPU_DATA_CORRUPT = -6
QZGPU_GPU_ERROR = -7
QZGPU_GPU_NOT_SUPPORTED = -8
QZGPU_GPU_NOT_ENOUGH_MEMORY = -9
QZGPU_TIMEOUT = -10
QZGPU_BLOCK_TOO_LARGE = -11
QZGPU_NOALLOC_MAX_BLOCK = 1 << 20

LIB_PATH = _build.LIB
_lock = threading.Lock()
_lib = None


class QzGpuError(RuntimeError):
    """A negative qzgpu return code (libbsc's error numbering, bsc.rs:17-24)."""

    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = error_string(code) if _lib is not None else str(code)
        super().__init__(f"{what} failed with error code {code} ({msg})")


class Stats(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_int), ("kernel_launches", ctypes.c_int),
                ("active_total", ctypes.c_longlong), ("alg_bytes", ctypes.c_longlong)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int), ("ms", ctypes.c_double),
                ("alg_bytes", ctypes.c_longlong)]


class StreamsInfo(ctypes.Structure):
    _fields_ = [("records", ctypes.c_longlong), ("header_bytes", ctypes.c_longlong),
                ("seq_bytes", ctypes.c_longlong), ("qual_bytes", ctypes.c_longlong),
                ("const_seq_len", ctypes.c_int), ("const_qual_len", ctypes.c_int),
                ("error_record", ctypes.c_longlong)]


_u8p = ctypes.POINTER(ctypes.c_uint8)
_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/qzgpu.h
SIGNATURES = {
    "qzgpu_init": (ctypes.c_int, [ctypes.c_int]),
    "qzgpu_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "qzgpu_bwt_encode": (ctypes.c_int, [_u8p, ctypes.c_int, _u8p, _i32p, ctypes.c_int]),
    "qzgpu_bwt_decode": (ctypes.c_int, [_u8p, ctypes.c_int, ctypes.c_int, ctypes.c_uint8, _i32p, ctypes.c_int]),
    "qzgpu_aux_rate": (ctypes.c_int, [ctypes.c_int]),
    "qzgpu_storage_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_longlong, ctypes.c_int]),
    "qzgpu_storage_destroy": (ctypes.c_int, [_vp]),
    "qzgpu_storage_bytes": (ctypes.c_longlong, [ctypes.c_longlong, ctypes.c_int]),
    "qzgpu_bwt_encode_batch": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_u8p), ctypes.POINTER(_u8p),
                                              _i32p, _i32p, ctypes.c_int]),
    "qzgpu_bwt_decode_batch": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_u8p), ctypes.POINTER(_u8p),
                                              _i32p, _i32p, ctypes.c_int]),
    "qzgpu_bwt_encode_device": (ctypes.c_int, [_vp, ctypes.c_int, _i32p, _vp, _vp, _i32p, _vp]),
    "qzgpu_bwt_decode_device": (ctypes.c_int, [_vp, ctypes.c_int, _i32p, _i32p, _vp, _vp, _vp]),
    "qzgpu_storage_last_stats": (ctypes.c_int, [_vp, ctypes.POINTER(Stats)]),
    "qzgpu_storage_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
    "qzgpu_storage_profile_only": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "qzgpu_fastq_streams": (ctypes.c_int, [_u8p, ctypes.c_longlong, _u8p, ctypes.c_longlong, _u8p, ctypes.c_longlong,
                                           _u8p, ctypes.c_longlong, _vp]),
    "qzgpu_storage_set_param": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_longlong]),
    "qzgpu_storage_get_param": (ctypes.c_longlong, [_vp, ctypes.c_char_p]),
    "qzgpu_bwt_decode_noalloc": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "qzgpu_server_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_longlong, ctypes.c_int, ctypes.c_longlong,
                                           ctypes.c_int]),
    "qzgpu_server_slots": (ctypes.c_int, [_vp]),
    "qzgpu_server_submit": (ctypes.c_longlong, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int]),
    "qzgpu_server_wait": (ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.c_int, _i32p, _i32p,
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "qzgpu_server_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "qzgpu_server_destroy": (ctypes.c_int, [_vp]),
    "qzgpu_storage_round_counts": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "qzgpu_storage_profile_read": (ctypes.c_int, [_vp, ctypes.POINTER(KernelTime), ctypes.c_int, ctypes.c_int]),
}


def load(build_if_missing: bool = True):
    """Loads the library (building it first if needed) and binds the C ABI."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise QzGpuError(QZGPU_GPU_NOT_SUPPORTED, f"loading {LIB_PATH} (not built)")
                _build.build()
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def error_string(code: int) -> str:
    return load().qzgpu_error_string(code).decode()


def check(rc: int, what: str) -> int:
    if rc < 0:
        raise QzGpuError(rc, what)
    return rc
