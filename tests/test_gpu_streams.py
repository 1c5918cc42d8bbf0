"""GPU stream building (qzgpu_fastq_streams) against the CPU oracle
(oracle/streams.py), bit-exact: byte work, no tolerance."""
import numpy as np
import pytest

from oracle import streams as S
from qz_gb300 import bwt, synth
from qz_gb300 import streams as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    bwt.init()
    return True


def _check(text):
    text = bytes(text)
    want = S.fastq_streams(text)
    h, s, q, info = G.fastq_streams(text)
    assert bytes(h) == want[0] and bytes(s) == want[1] and bytes(q) == want[2]
    assert info["records"] == want[3]
    assert info["const_seq_len"] == want[4] and info["const_qual_len"] == want[5]
    assert info["error_record"] == -1
    return h, s, q, info


def test_chunk_matches_oracle_and_synth(gpu):
    n = 20_000
    text = synth.chunk_fastq(n)
    h, s, q, info = _check(text)
    g = synth.uniform_genome(5_000_000, seed=1)
    assert (s == synth.sample_reads(g, n, seed=2)).all()
    assert (q == synth.quality_stream(n, seed=3)).all()
    assert (h == synth.header_stream(n, seed=4)).all()


def test_variable_lengths(gpu):
    rng = np.random.default_rng(7)
    parts = []
    for r in range(3000):
        L = int(rng.integers(0, 400))
        seq = bytes(rng.choice(list(b"ACGTN"), L).astype(np.uint8))
        qual = bytes(rng.integers(30, 200, L).astype(np.uint8))  # below '!' and above 127 + 33
        rid = b"@r%d" % r + b"x" * int(rng.integers(0, 300))      # ids past 127 bytes: 2-byte varints
        parts.append(rid + b"\n" + seq + b"\n+" + b"c" * int(r % 3) + b"\n" + qual + b"\n")
    _check(b"".join(parts))


def test_crlf_and_no_final_newline(gpu):
    _check(b"@r1\r\nACG\r\n+\r\n!!I\r\n@r2\r\nTTT\r\n+\r\nIII")
    _check(b"@r1\nACG\n+\n!!I\n@r2\nTTT\n+\nIII")


def test_empty_and_tiny(gpu):
    h, s, q, info = G.fastq_streams(b"")
    assert len(h) == len(s) == len(q) == 0 and info["records"] == 0
    _check(b"@\n\n+\n\n")
    _check(b"@a\nA\n+\nI\n")


@pytest.mark.parametrize("text,rec", [
    (b"@a\nACGT\n-\nIIII\n", 0),
    (b"@a\nACGT\n+\nIII\n", 0),
    (b"@a\nACGT\n+\nIIII\n@b\nAC\n", 1),
    (b"@a\nACGT\n+\nIIII\n@b\nAC\n+\n", 1),
    (b"@a\nACGT\n+\nIIII\n\n", 1),
    (b"@a\nACGT\n+\nIIII\n@b\nAC\n-\nII\n@c\nA\n+\nI\n", 1),
    (b"single line without newline", 0),
])
def test_malformed_matches_reader(gpu, text, rec):
    with pytest.raises(S.FastqError) as e:
        S.fastq_streams(text)
    assert e.value.record == rec
    with pytest.raises(G.FastqError) as g:
        G.fastq_streams(text)
    assert g.value.record == rec


def test_reused_outputs_and_sizes(gpu):
    text = synth.chunk_fastq(2000)
    h0, s0, q0, info = G.fastq_streams(text)
    out = (np.empty(info["header_bytes"], np.uint8), np.empty(info["seq_bytes"], np.uint8),
           np.empty(info["qual_bytes"], np.uint8))
    for _ in range(2):
        h, s, q, _ = G.fastq_streams(text, out=out)
        assert (h == h0).all() and (s == s0).all() and (q == q0).all()
    small = (out[0][:-1], out[1], out[2])
    with pytest.raises(bwt.native.QzGpuError):
        G.fastq_streams(text, out=small)
