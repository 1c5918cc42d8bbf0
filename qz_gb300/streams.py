"""Host API of the device stream builder (qzgpu_fastq_streams): FASTQ text in,
qz's header / sequence / quality streams out, as records_to_streams builds
them on qz's default lossless BSC path (crates/qz-lib/src/compression/
mod.rs:270-325, columnar.rs:104-134, io/fastq.rs:135-200)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .native import QzGpuError

_u8p = ctypes.POINTER(ctypes.c_uint8)


class FastqError(QzGpuError):
    """Malformed FASTQ: `record` is the record the reader fails on."""

    def __init__(self, code: int, record: int):
        super().__init__(code, f"qzgpu_fastq_streams: malformed FASTQ at record {record}")
        self.record = record


def _info_dict(info: native.StreamsInfo) -> dict:
    return {k: getattr(info, k) for k, _ in native.StreamsInfo._fields_}


def fastq_streams(text, out=None):
    """(header stream, sequence stream, quality stream, info) of FASTQ text.
    `out`: optional (header, seq, qual) uint8 arrays large enough, reused by
    streaming callers.  Raises FastqError for malformed input."""
    t = np.frombuffer(text, dtype=np.uint8) if isinstance(text, (bytes, bytearray, memoryview)) else \
        np.ascontiguousarray(text, dtype=np.uint8)
    L = native.load()
    info = native.StreamsInfo()
    buf = t if len(t) else np.zeros(1, np.uint8)
    n = len(t)
    if out is None:
        rc = L.qzgpu_fastq_streams(buf.ctypes.data_as(_u8p), n, None, 0, None, 0, None, 0, ctypes.byref(info))
        if rc == native.QZGPU_DATA_CORRUPT:
            raise FastqError(rc, info.error_record)
        if rc not in (0, native.QZGPU_BAD_PARAMETER):
            native.check(rc, "qzgpu_fastq_streams")
        out = (np.empty(max(info.header_bytes, 1), np.uint8), np.empty(max(info.seq_bytes, 1), np.uint8),
               np.empty(max(info.qual_bytes, 1), np.uint8))
    h, s, q = out
    rc = L.qzgpu_fastq_streams(buf.ctypes.data_as(_u8p), n, h.ctypes.data_as(_u8p), len(h), s.ctypes.data_as(_u8p),
                               len(s), q.ctypes.data_as(_u8p), len(q), ctypes.byref(info))
    if rc == native.QZGPU_DATA_CORRUPT:
        raise FastqError(rc, info.error_record)
    native.check(rc, "qzgpu_fastq_streams")
    return h[: info.header_bytes], s[: info.seq_bytes], q[: info.qual_bytes], _info_dict(info)
