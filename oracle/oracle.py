"""ctypes wrapper over the C oracle (oracle/bwt_oracle.c).

Test infrastructure only: tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` import this module as the checker.  The product
path (``qz_gb300``) never imports it.

Parity status: unpinned against libbsc (its source is not in the reference
tree); pinned against the brute-force definition and textbook known answers.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
# the same source built with the reference's kind of flags (-O3, host core
# tuning); only the benchmark's timed CPU baseline loads it
_TUNED_PATH = os.path.join(_HERE, "_build", "liboracle_tuned.so")
_lock = threading.Lock()
_libs = {}

PRIMARY_INDEX_OFFSET = 1


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, portable flags)."""
    src = os.path.getmtime(os.path.join(_HERE, "bwt_oracle.c"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (_LIB_PATH, _TUNED_PATH)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib(tuned: bool = False):
    with _lock:
        key = "tuned" if tuned else "portable"
        if key not in _libs:
            build()
            L = ctypes.CDLL(_TUNED_PATH if tuned else _LIB_PATH)
            u8p = ctypes.POINTER(ctypes.c_uint8)
            i32p = ctypes.POINTER(ctypes.c_int32)
            L.oracle_suffix_array.argtypes = [u8p, i32p, ctypes.c_int32]
            L.oracle_suffix_array_bruteforce.argtypes = [u8p, i32p, ctypes.c_int32]
            L.oracle_suffix_array_doubling.argtypes = [u8p, i32p, ctypes.c_int32]
            L.oracle_bwt_encode.argtypes = [u8p, u8p, ctypes.c_int32, ctypes.c_int32, i32p]
            L.oracle_bwt_decode.argtypes = [u8p, u8p, ctypes.c_int32, ctypes.c_int32]
            L.oracle_bwt_batch.argtypes = [
                ctypes.c_int, ctypes.c_int32, ctypes.POINTER(u8p), ctypes.POINTER(u8p), i32p, i32p, i32p,
                ctypes.c_int32,
            ]
            for f in (L.oracle_suffix_array, L.oracle_suffix_array_bruteforce, L.oracle_suffix_array_doubling,
                      L.oracle_bwt_encode,
                      L.oracle_bwt_decode, L.oracle_bwt_batch):
                f.restype = ctypes.c_int
            _libs[key] = L
    return _libs[key]


def _u8(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _i32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def as_u8(data) -> np.ndarray:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(data), dtype=np.uint8).copy()
    return np.ascontiguousarray(data, dtype=np.uint8)


def suffix_array(data, brute: bool = False, method: str = "sais") -> np.ndarray:
    """Suffix array with an implicit smallest end sentinel.  method: "sais"
    (induced sorting), "doubling" (prefix doubling) or "brute" (direct
    comparison, small inputs); brute=True is the same as method="brute"."""
    t = as_u8(data)
    sa = np.empty(max(len(t), 1), dtype=np.int32)
    if brute:
        method = "brute"
    f = {"sais": lib().oracle_suffix_array, "doubling": lib().oracle_suffix_array_doubling,
         "brute": lib().oracle_suffix_array_bruteforce}[method]
    rc = f(_u8(t), _i32(sa), len(t))
    if rc:
        raise RuntimeError(f"oracle suffix array failed: {rc}")
    return sa[: len(t)]


def bwt_encode(data, aux_rate: int = 0):
    """Forward BWT. Returns (U, primary_index) or (U, primary_index, aux) when aux_rate > 0."""
    t = as_u8(data)
    n = len(t)
    u = np.empty(max(n, 1), dtype=np.uint8)
    aux = np.zeros(((n - 1) // aux_rate + 1) if (aux_rate and n) else 1, dtype=np.int32)
    rc = lib().oracle_bwt_encode(_u8(t), _u8(u), n, aux_rate, _i32(aux) if aux_rate else None)
    if rc < 0:
        raise RuntimeError(f"oracle bwt encode failed: {rc}")
    if aux_rate:
        return u[:n], rc, aux
    return u[:n], rc


def bwt_decode(u, index: int) -> np.ndarray:
    u = as_u8(u)
    n = len(u)
    t = np.empty(max(n, 1), dtype=np.uint8)
    rc = lib().oracle_bwt_decode(_u8(u), _u8(t), n, int(index))
    if rc:
        raise ValueError(f"oracle bwt decode failed: {rc}")
    return t[:n]


def _batch(direction: int, blocks, index=None, threads: int | None = None, tuned: bool = False):
    blocks = [as_u8(b) for b in blocks]
    nb = len(blocks)
    outs = [np.empty(max(len(b), 1), dtype=np.uint8) for b in blocks]
    u8p = ctypes.POINTER(ctypes.c_uint8)
    inp = (u8p * max(nb, 1))(*[_u8(b) for b in blocks])
    outp = (u8p * max(nb, 1))(*[_u8(o) for o in outs])
    ns = np.array([len(b) for b in blocks] or [0], dtype=np.int32)
    idx = np.array(index if index is not None else [0] * nb, dtype=np.int32) if nb else np.zeros(1, np.int32)
    st = np.zeros(max(nb, 1), dtype=np.int32)
    threads = threads or os.cpu_count() or 1
    rc = lib(tuned).oracle_bwt_batch(direction, nb, inp, outp, _i32(ns), _i32(idx), _i32(st), threads)
    if rc < 0:
        raise RuntimeError(f"oracle batch failed: {rc}")
    return [o[: len(b)] for o, b in zip(outs, blocks)], idx[:nb]


def bwt_encode_batch(blocks, threads: int | None = None, tuned: bool = False):
    """Forward BWT of many blocks over host threads, one block per thread at a
    time; returns (list of U, indexes).  tuned: the -O3 host-tuned build."""
    return _batch(0, blocks, None, threads, tuned)


def bwt_decode_batch(blocks, indexes, threads: int | None = None, tuned: bool = False):
    outs, _ = _batch(1, blocks, list(indexes), threads, tuned)
    return outs


def naive_bwt(data) -> tuple[bytes, int]:
    """Definition-level BWT in pure Python (tiny inputs): sort all suffixes with
    an implicit smallest end marker, then apply the output convention."""
    t = bytes(data)
    n = len(t)
    if n == 0:
        return b"", 0
    order = sorted(range(n), key=lambda i: t[i:])
    out = bytearray([t[n - 1]])
    primary = -1
    for j, p in enumerate(order):
        if p == 0:
            primary = j + PRIMARY_INDEX_OFFSET
        else:
            out.append(t[p - 1])
    return bytes(out), primary
