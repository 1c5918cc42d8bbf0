"""The seeded synthetic workloads have the shapes the benchmark configurations
name (no GPU): block sizes, stream layouts and value distributions of qz's
sequence, quality and header streams."""
import re

import numpy as np
import pytest

from qz_gb300 import synth

HEADER_RE = re.compile(rb"^@SIM:1:FC01:([1-4]):(\d+):(\d+):(\d+) 1:N:0:[ACGT]{8}$")


def _unpack_qualities(stream, nreads, read_len=150):
    per = (read_len * 7 + 7) // 8
    bits = np.unpackbits(stream[: nreads * per].reshape(nreads, per), axis=1, bitorder="little")
    bits = bits[:, : read_len * 7].reshape(nreads, read_len, 7)
    return (bits << np.arange(7, dtype=np.uint8)).sum(axis=2).astype(np.uint8)


def test_plain_block_shape():
    b = synth.plain_block()
    assert len(b) == 24_999_900  # 166,666 x 150 bp, constant length: no varints
    counts = np.bincount(b, minlength=256)
    assert set(np.nonzero(counts)[0]) <= set(b"ACGTN")
    assert 0 < counts[ord("N")] / len(b) < 5e-4  # 0.01% N


def test_chunk_stream_cut():
    # 2.5M reads: 375,000,000 sequence bytes cut into 25 MiB blocks (14 full + 7,998,400)
    blocks = synth.cut_blocks(np.empty(375_000_000, dtype=np.uint8))
    assert [len(b) for b in blocks] == [26_214_400] * 14 + [7_998_400]
    # qualities: 132 packed bytes per 150 bp read -> 330,000,000 bytes, 13 blocks
    assert len(synth.cut_blocks(np.empty(2_500_000 * 132, dtype=np.uint8))) == 13


def test_quality_stream_model():
    n = 20_000
    s = synth.quality_stream(n, seed=3)
    assert len(s) == n * 132  # 7 bits per value, padded per read
    q = _unpack_qualities(s, n)
    assert np.array_equal(q, synth.quality_values(n, seed=3))
    assert set(np.unique(q)) <= {2, 12, 23, 37}
    # the per-read chain leaves its state with probability 1 - stay, stay
    # falling linearly from 0.95 to 0.80 along the read
    change = (q[:, 1:] != q[:, :-1]).mean(axis=0)
    assert change[:10].mean() == pytest.approx(0.05, abs=0.01)
    assert change[-10:].mean() == pytest.approx(0.20, abs=0.015)


def test_header_ids_and_stream():
    n = 5_000
    ids = synth.header_ids(n, seed=4)
    last = {}
    for i in ids:
        m = HEADER_RE.match(i)
        assert m, i
        lane, tile, x = int(m.group(1)), int(m.group(2)), int(m.group(3))
        assert 1101 <= tile <= 2624 and 1 <= x <= 32000
        # x increases within each tile
        assert x >= last.get((lane, tile), 0)
        last[(lane, tile)] = x
    s = synth.header_stream(n, seed=4).tobytes()
    # [varint(len)][id] per read; every id here is shorter than 128 bytes
    pos = 0
    for i in ids:
        assert s[pos] == len(i) and s[pos + 1:pos + 1 + len(i)] == i
        pos += 1 + len(i)
    assert pos == len(s)


def test_uneven_batch_shape():
    blocks = synth.uneven_blocks(max_source=3_000_000)
    assert len(blocks) == 256
    kinds = [k for k, _ in blocks]
    assert kinds.count("dna") / 256 == pytest.approx(0.5, abs=0.1)
    assert kinds.count("qual") / 256 == pytest.approx(0.3, abs=0.1)
    assert kinds.count("hdr") / 256 == pytest.approx(0.2, abs=0.1)
    sizes = np.array([len(b) for _, b in blocks])
    assert sizes.min() >= 1024 and sizes.max() <= synth.BLOCK_BYTES
    # log-uniform: about half the blocks below the geometric midpoint (~164 KB)
    assert (sizes < np.sqrt(1024 * synth.BLOCK_BYTES)).mean() == pytest.approx(0.5, abs=0.12)


def test_repeat_blocks_shape():
    blocks = synth.repeat_blocks()
    assert [k for k, _ in blocks] == ["repeat", "repeat", "single", "period3"]
    assert [len(b) for _, b in blocks] == [26_214_400, 3_785_600, 26_214_400, 26_214_400]
    assert (blocks[2][1] == ord("A")).all()
    assert bytes(blocks[3][1][:6]) == b"ACGACG"
