"""CPU: the stream-building oracle (oracle/streams.py) against the independent
stream builders of qz_gb300.synth, and the reader's edge cases."""
import numpy as np
import pytest

from oracle import streams as S
from qz_gb300 import synth


def test_oracle_matches_synth_streams():
    n = 3000
    g = synth.uniform_genome(5_000_000, seed=1)
    text = synth.chunk_fastq(n)
    hdr, seq, qual, recs, cs, cq = S.fastq_streams(text.tobytes())
    assert recs == n and cs == 150 and cq == 150
    assert seq == synth.sample_reads(g, n, seed=2).tobytes()
    assert qual == synth.quality_stream(n, seed=3).tobytes()
    assert hdr == synth.header_stream(n, seed=4).tobytes()


def test_variable_lengths_write_varints():
    text = b"@a\nACGT\n+\nIIII\n@bb\nAC\n+x\nI#\n"
    hdr, seq, qual, recs, cs, cq = S.fastq_streams(text)
    assert recs == 2 and cs == 0 and cq == 0
    assert hdr == b"\x02@a\x03@bb"
    assert seq == b"\x04ACGT\x02AC"
    assert qual == b"\x04" + S.pack_qualities(b"IIII") + b"\x02" + S.pack_qualities(b"I#")


def test_crlf_and_missing_final_newline():
    a = S.fastq_streams(b"@r1\r\nACG\r\n+\r\n!!I\r\n@r2\r\nTTT\r\n+\r\nIII")
    b = S.fastq_streams(b"@r1\nACG\n+\n!!I\n@r2\nTTT\n+\nIII\n")
    assert a == b


def test_quality_saturation_and_packing():
    # below '!' saturates to 0, above 127 + 33 clips to 127; 7 bits LSB first
    # bits: 0 @0-6, 0 @7-13, 1 @14-20, 127 @21-27
    assert S.pack_qualities(bytes([10, 33, 34, 200])) == bytes([0x00, 0x40, 0xE0, 0x0F])
    assert len(S.pack_qualities(b"I" * 150)) == 132


def test_long_id_two_byte_varint():
    rid = b"@" + b"x" * 200
    hdr = S.fastq_streams(rid + b"\nA\n+\nI\n")[0]
    assert hdr[:2] == bytes([201 & 0x7F | 0x80, 201 >> 7]) and hdr[2:] == rid


def test_empty_input():
    assert S.fastq_streams(b"") == (b"", b"", b"", 0, 0, 0)


@pytest.mark.parametrize("text,rec", [
    (b"@a\nACGT\n-\nIIII\n", 0),                # separator not '+'
    (b"@a\nACGT\n+\nIII\n", 0),                 # length mismatch
    (b"@a\nACGT\n+\nIIII\n@b\nAC\n", 1),        # EOF at the separator
    (b"@a\nACGT\n+\nIIII\n@b\nAC\n+\n", 1),     # EOF at the quality line
    (b"@a\nACGT\n+\nIIII\n\n", 1),              # trailing blank line
])
def test_malformed(text, rec):
    with pytest.raises(S.FastqError) as e:
        S.fastq_streams(text)
    assert e.value.record == rec
