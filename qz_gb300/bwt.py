"""Python host API over the C ABI: the calls qz's BSC wrapper makes, one block
or many, on host or device buffers.

Mirrors the block surface of crates/qz-lib/src/compression/bsc.rs: empty input
short-circuits before the library is called (bsc.rs:162-164, 387-389), sizes
above c_int::MAX are rejected (bsc.rs:165-167), and any negative library code
raises (bsc.rs:185-187, 411-433 turn them into anyhow errors).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .native import QzGpuError, check

_u8p = ctypes.POINTER(ctypes.c_uint8)
_i32p = ctypes.POINTER(ctypes.c_int32)
C_INT_MAX = 2**31 - 1


def _as_u8(data) -> np.ndarray:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(data), dtype=np.uint8).copy()
    return np.array(data, dtype=np.uint8, copy=True)


def _view_u8(data) -> np.ndarray:
    """Contiguous uint8 view of a caller's buffer (a copy only when needed)."""
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(data, dtype=np.uint8)
    return np.ascontiguousarray(data, dtype=np.uint8)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u8p)


def init() -> None:
    check(native.load().qzgpu_init(0), "qzgpu_init")


def aux_rate(n: int) -> int:
    return native.load().qzgpu_aux_rate(int(n))


def bwt_encode(data, with_aux: bool = False):
    """Forward BWT of one block (libbsc's bsc_bwt_encode semantics).

    Returns (U, primary_index) or (U, primary_index, aux_indexes)."""
    t = _as_u8(data)
    n = len(t)
    if n > C_INT_MAX:
        raise QzGpuError(native.QZGPU_BAD_PARAMETER, f"BSC input too large: {n} bytes")
    L = native.load()
    num = ctypes.c_uint8(0)
    aux = np.zeros(256, dtype=np.int32)
    buf = t if n else np.zeros(1, np.uint8)
    rc = L.qzgpu_bwt_encode(_ptr(buf), n, ctypes.cast(ctypes.pointer(num), _u8p) if with_aux else None,
                            aux.ctypes.data_as(_i32p) if with_aux else None, 0)
    check(rc, "qzgpu_bwt_encode")
    if with_aux:
        return t, rc, aux[: num.value].copy()
    return t, rc


def bwt_decode(u, index: int) -> np.ndarray:
    """Inverse BWT of one block (libbsc's bsc_bwt_decode semantics)."""
    t = _as_u8(u)
    n = len(t)
    buf = t if n else np.zeros(1, np.uint8)
    check(native.load().qzgpu_bwt_decode(_ptr(buf), n, int(index), 0, None, 0), "qzgpu_bwt_decode")
    return t


class Storage:
    """Device scratch for batches of up to ``max_total_bytes`` bytes in
    ``max_blocks`` blocks (libcubwt-style: allocate once, reuse)."""

    def __init__(self, max_total_bytes: int, max_blocks: int = 1):
        self._lib = native.load()
        h = ctypes.c_void_p()
        check(self._lib.qzgpu_storage_create(ctypes.byref(h), int(max_total_bytes), int(max_blocks)),
              "qzgpu_storage_create")
        self._h = h
        self.max_total_bytes = int(max_total_bytes)
        self.max_blocks = int(max_blocks)

    @staticmethod
    def device_bytes(max_total_bytes: int, max_blocks: int) -> int:
        return native.load().qzgpu_storage_bytes(int(max_total_bytes), int(max_blocks))

    def close(self) -> None:
        if self._h:
            self._lib.qzgpu_storage_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self) -> dict:
        s = native.Stats()
        check(self._lib.qzgpu_storage_last_stats(self._h, ctypes.byref(s)), "qzgpu_storage_last_stats")
        return {"rounds": s.rounds, "kernel_launches": s.kernel_launches, "active_total": s.active_total,
                "alg_bytes": s.alg_bytes}

    PARAMS = ("fwd_sub_bytes", "inv_sub_bytes", "big_ctas_per_sm", "tile_ctas_per_sm", "medium_max",
              "ruler_stride_log2", "big_tile", "radix_first_bits", "round_pipeline", "split_lookback",
              "rank_mode", "early_counts", "pass0_bulk")

    def set_param(self, name: str, value: int) -> None:
        check(self._lib.qzgpu_storage_set_param(self._h, name.encode(), int(value)), f"set_param({name})")

    def get_param(self, name: str) -> int:
        return check(self._lib.qzgpu_storage_get_param(self._h, name.encode()), f"get_param({name})")

    def params(self) -> dict:
        return {k: self.get_param(k) for k in self.PARAMS + ("lanes",)}

    def round_counts(self) -> list[int]:
        """Suffixes sorted per round of the last forward call (entry 0 = all)."""
        buf = (ctypes.c_longlong * 64)()
        n = check(self._lib.qzgpu_storage_round_counts(self._h, buf, 64), "qzgpu_storage_round_counts")
        return [int(buf[i]) for i in range(min(n, 64))]

    def profile(self, enable: bool = True, only: str | None = None) -> None:
        """Times every later launch on this storage with CUDA events (only the
        launches of kernel `only` when it is given)."""
        check(self._lib.qzgpu_storage_profile_only(self._h, (only or "").encode()), "qzgpu_storage_profile_only")
        check(self._lib.qzgpu_storage_profile(self._h, int(enable)), "qzgpu_storage_profile")

    def profile_read(self, reset: bool = True) -> list[dict]:
        buf = (native.KernelTime * 64)()
        n = check(self._lib.qzgpu_storage_profile_read(self._h, buf, 64, int(reset)), "qzgpu_storage_profile_read")
        return [{"name": buf[i].name.decode(), "launches": buf[i].launches, "ms": buf[i].ms,
                 "alg_bytes": buf[i].alg_bytes} for i in range(min(n, 64))]

    def _ptr_arrays(self, ins, outs):
        nb = len(ins)
        inp = (_u8p * max(nb, 1))(*[_ptr(b) for b in ins])
        outp = (_u8p * max(nb, 1))(*[_ptr(b) for b in outs])
        return inp, outp

    @staticmethod
    def _outs(sizes, out):
        if out is None:
            return [np.empty(max(int(n), 1), np.uint8) for n in sizes]
        if len(out) != len(sizes):
            raise QzGpuError(native.QZGPU_BAD_PARAMETER, "out: one buffer per block")
        outs = []
        for n, o in zip(sizes, out):
            if not (isinstance(o, np.ndarray) and o.dtype == np.uint8 and o.flags.c_contiguous and o.flags.writeable
                    and len(o) >= n):
                raise QzGpuError(native.QZGPU_BAD_PARAMETER, "out: writable contiguous uint8 arrays of block size")
            outs.append(o if n else np.zeros(1, np.uint8))
        return outs

    def encode_batch(self, blocks, out=None):
        """Forward BWT of many blocks in one batched launch sequence.
        Returns (list of U, list of primary indexes).  `out`: optional output
        arrays, one per block (reused across calls by streaming callers)."""
        ins = [_view_u8(b) for b in blocks]
        ins = [b if len(b) else np.zeros(1, np.uint8) for b in ins]
        sizes = np.array([len(b) for b in blocks] or [0], dtype=np.int32)
        outs = self._outs([len(b) for b in blocks], out)
        idx = np.zeros(max(len(blocks), 1), dtype=np.int32)
        inp, outp = self._ptr_arrays(ins, outs)
        check(self._lib.qzgpu_bwt_encode_batch(self._h, len(blocks), inp, outp, sizes.ctypes.data_as(_i32p),
                                               idx.ctypes.data_as(_i32p), 0), "qzgpu_bwt_encode_batch")
        return [o[: s] for o, s in zip(outs, sizes)], [int(i) for i in idx[: len(blocks)]]

    def decode_batch(self, blocks, indexes, out=None):
        """Inverse BWT of many blocks; `out` as for encode_batch."""
        ins = [_view_u8(b) for b in blocks]
        ins = [b if len(b) else np.zeros(1, np.uint8) for b in ins]
        sizes = np.array([len(b) for b in blocks] or [0], dtype=np.int32)
        outs = self._outs([len(b) for b in blocks], out)
        idx = np.array(list(indexes) or [0], dtype=np.int32)
        inp, outp = self._ptr_arrays(ins, outs)
        check(self._lib.qzgpu_bwt_decode_batch(self._h, len(blocks), inp, outp, sizes.ctypes.data_as(_i32p),
                                               idx.ctypes.data_as(_i32p), 0), "qzgpu_bwt_decode_batch")
        return [o[: s] for o, s in zip(outs, sizes)]

    def encode_device(self, sizes, d_T: int, d_U: int, stream: int = 0):
        """Device buffers (blocks back to back) -> list of primary indexes."""
        sz = np.array(list(sizes) or [0], dtype=np.int32)
        idx = np.zeros(max(len(sizes), 1), dtype=np.int32)
        check(self._lib.qzgpu_bwt_encode_device(self._h, len(sizes), sz.ctypes.data_as(_i32p), ctypes.c_void_p(d_T),
                                                ctypes.c_void_p(d_U), idx.ctypes.data_as(_i32p),
                                                ctypes.c_void_p(stream)), "qzgpu_bwt_encode_device")
        return [int(i) for i in idx[: len(sizes)]]

    def decode_device(self, sizes, indexes, d_U: int, d_T: int, stream: int = 0) -> None:
        sz = np.array(list(sizes) or [0], dtype=np.int32)
        idx = np.array(list(indexes) or [0], dtype=np.int32)
        check(self._lib.qzgpu_bwt_decode_device(self._h, len(sizes), sz.ctypes.data_as(_i32p),
                                                idx.ctypes.data_as(_i32p), ctypes.c_void_p(d_U),
                                                ctypes.c_void_p(d_T), ctypes.c_void_p(stream)),
              "qzgpu_bwt_decode_device")


class Server:
    """Serving form over the C ABI: requests from any thread are batched
    continuously onto device-resident slots (qzgpu_server_*)."""

    FORWARD = 0
    INVERSE = 1

    def __init__(self, hbm_budget: int = 0, max_slots: int = 4, slot_bytes: int = 0, slot_blocks: int = 0):
        import threading

        self._lib = native.load()
        h = ctypes.c_void_p()
        check(self._lib.qzgpu_server_create(ctypes.byref(h), int(hbm_budget), int(max_slots), int(slot_bytes),
                                            int(slot_blocks)), "qzgpu_server_create")
        self._h = h
        self._bufs = {}
        self._lock = threading.Lock()

    @property
    def slots(self) -> int:
        """Slots the server holds now (it admits more under load, by free HBM)."""
        return check(self._lib.qzgpu_server_slots(self._h), "qzgpu_server_slots")

    def _submit(self, op: int, data, index: int) -> int:
        src = _as_u8(data)
        n = len(src)
        if n == 0:
            src = np.zeros(1, np.uint8)
        out = np.empty(max(n, 1), np.uint8)
        t = self._lib.qzgpu_server_submit(self._h, op, src.ctypes.data_as(ctypes.c_void_p),
                                          out.ctypes.data_as(ctypes.c_void_p), n, int(index))
        check(t, "qzgpu_server_submit")
        with self._lock:
            self._bufs[t] = (src, out, n)
        return t

    def submit_forward(self, block) -> int:
        return self._submit(self.FORWARD, block, 0)

    def submit_inverse(self, u, index: int) -> int:
        return self._submit(self.INVERSE, u, index)

    def wait(self, ticket: int, timeout_ms: int = -1):
        st = ctypes.c_int32(0)
        ix = ctypes.c_int32(0)
        lat = ctypes.c_double(0)
        q = ctypes.c_double(0)
        rc = self._lib.qzgpu_server_wait(self._h, int(ticket), int(timeout_ms), ctypes.byref(st), ctypes.byref(ix),
                                         ctypes.byref(lat), ctypes.byref(q))
        check(rc, "qzgpu_server_wait")
        if rc == 0:
            return None
        with self._lock:
            src, out, n = self._bufs.pop(ticket)
        check(st.value, "served request")
        return {"out": out[:n], "index": ix.value, "latency_ms": lat.value, "queue_ms": q.value}

    def stats(self) -> dict:
        buf = (ctypes.c_longlong * 7)()
        check(self._lib.qzgpu_server_stats(self._h, buf, 7), "qzgpu_server_stats")
        keys = ("completed", "batches", "max_batch", "max_slots_busy", "waiting", "slots", "admission_refused")
        return dict(zip(keys, (int(v) for v in buf)))

    def close(self) -> None:
        if self._h:
            self._lib.qzgpu_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
