"""The allocation-free inverse BWT (qzgpu_bwt_decode_noalloc) against the
existing inverse entry point, through the C ABI.

This entry point serves callers that cannot allocate device memory while they
run, for example a host runtime that hands out all device memory up front and
forbids later cudaMalloc/cudaFree.  Its scratch is a fixed device array shared
by every call, so two calls in a row must both give the existing entry point's
output (bit-exact: byte work has no tolerance).  This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

from qz_gb300 import bwt, native, synth

pytestmark = pytest.mark.gpu


def _noalloc(lib, d_u, d_t, n, index, stream):
    return lib.qzgpu_bwt_decode_noalloc(ctypes.c_void_p(d_u), ctypes.c_void_p(d_t), int(n), int(index),
                                        ctypes.c_void_p(stream))


def test_noalloc_decode_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    lib = native.load()
    bwt.init()
    stream = torch.cuda.current_stream().cuda_stream
    blocks = [
        synth.sample_reads(synth.uniform_genome(60_000, seed=61), 2000, seed=62),  # 300,000 bytes of DNA
        synth.quality_stream(8000, seed=63)[: native.QZGPU_NOALLOC_MAX_BLOCK],    # the 1 MiB limit exactly
    ]
    for t in blocks:  # two calls in a row share the scratch array
        u, idx = bwt.bwt_encode(t)
        expected = bwt.bwt_decode(u, idx)  # existing entry point
        d_u = torch.from_numpy(np.ascontiguousarray(u)).cuda()
        d_t = torch.empty_like(d_u)
        rc = _noalloc(lib, d_u.data_ptr(), d_t.data_ptr(), len(u), idx, stream)
        assert rc == native.QZGPU_NO_ERROR, native.error_string(rc)
        torch.cuda.synchronize()
        assert np.array_equal(d_t.cpu().numpy(), expected)
        assert np.array_equal(expected, t)


def test_noalloc_rejects_blocks_over_the_limit():
    torch = pytest.importorskip("torch")
    lib = native.load()
    bwt.init()
    n = native.QZGPU_NOALLOC_MAX_BLOCK + 1
    d = torch.zeros(n, dtype=torch.uint8, device="cuda")
    rc = _noalloc(lib, d.data_ptr(), d.data_ptr(), n, 1, torch.cuda.current_stream().cuda_stream)
    assert rc == native.QZGPU_BLOCK_TOO_LARGE
    assert "larger" in native.error_string(rc)


def test_noalloc_in_place_and_large_then_small():
    # d_T may be d_U (in place), and a small block after a full-size one must
    # not see the larger call's leftovers in the shared scratch (sizes that are
    # not multiples of the 4096-byte tiles or the 32-row ruler stride)
    torch = pytest.importorskip("torch")
    lib = native.load()
    bwt.init()
    stream = torch.cuda.current_stream().cuda_stream
    g = synth.uniform_genome(80_000, seed=64)
    blocks = [synth.header_stream(30_000, seed=65)[: native.QZGPU_NOALLOC_MAX_BLOCK],
              synth.sample_reads(g, 40, seed=66)[:5_997],
              synth.quality_stream(300, seed=67)[:4_099],
              np.frombuffer(b"ab", np.uint8).copy()]
    for t in blocks:
        u, idx = bwt.bwt_encode(t)
        expected = bwt.bwt_decode(u, idx)  # existing entry point
        d = torch.from_numpy(np.ascontiguousarray(u)).cuda()
        rc = _noalloc(lib, d.data_ptr(), d.data_ptr(), len(u), idx, stream)
        assert rc == native.QZGPU_NO_ERROR, native.error_string(rc)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), expected)
        assert np.array_equal(expected, t)


def test_noalloc_one_byte_and_wrong_index():
    # a 1-byte block is its own transform; a wrong but in-range index gives
    # the existing entry point's answer (the same bytes, or the same
    # corrupt-data error), and the call returns either way
    torch = pytest.importorskip("torch")
    lib = native.load()
    bwt.init()
    stream = torch.cuda.current_stream().cuda_stream
    one = torch.tensor([0x41], dtype=torch.uint8, device="cuda")
    out = torch.zeros_like(one)
    rc = _noalloc(lib, one.data_ptr(), out.data_ptr(), 1, 1, stream)
    assert rc == native.QZGPU_NO_ERROR, native.error_string(rc)
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0x41]

    t = synth.sample_reads(synth.uniform_genome(5000, seed=53), 50, seed=54)
    u, idx = bwt.bwt_encode(t)
    wrong = idx % len(t) + 1
    try:
        expected, want_rc = bwt.bwt_decode(u, wrong), native.QZGPU_NO_ERROR
    except native.QzGpuError as e:
        expected, want_rc = None, e.code
    d_u = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    d_t = torch.empty_like(d_u)
    rc = _noalloc(lib, d_u.data_ptr(), d_t.data_ptr(), len(u), wrong, stream)
    torch.cuda.synchronize()
    assert rc == want_rc, (native.error_string(rc), want_rc)
    if rc == native.QZGPU_NO_ERROR:
        assert np.array_equal(d_t.cpu().numpy(), expected)
