"""CPU oracle for qz's stream building (test infrastructure only: the tests,
smoke() and the bench's CPU baseline use it as the checker; the library never
calls it).

Restates, record by record, what qz does to a FASTQ chunk before the block
sorter on its default lossless BSC path:

* FastqReader::next (crates/qz-lib/src/io/fastq.rs:135-200): four lines per
  record read up to and including '\\n'; trailing '\\n' / '\\r' trimmed from
  the id, sequence and quality lines; the separator line must start with '+';
  sequence and quality lengths must match; EOF at the separator or quality
  line is an error; EOF at an id line ends the input.
* detect_const_lengths (compression/mod.rs:329-354): a length is constant
  when every record has the first record's length.
* records_to_streams (compression/mod.rs:270-325) with quality mode lossless,
  no hints, no delta, no reverse-complement canonicalisation:
  header stream  [varint(len(id))][id];
  sequence stream [varint(len) if lengths vary][bases];
  quality stream  [varint(len) if lengths vary][pack_qualities(q, None)].
* pack_qualities with binning None (compression/columnar.rs:16-36, 104-134):
  phred = max(q - 33, 0), encoded = min(phred, 127), 7 bits each, LSB first,
  the last partial byte of each read flushed.
* write_varint (compression/mod.rs:683-689): 7 bits per byte, low first, high
  bit set on every byte but the last.

Parity unpinned against the reference itself (Rust, no toolchain here); the
tests cross-check this restatement against the independent stream builders of
qz_gb300.synth.
"""
from __future__ import annotations


class FastqError(ValueError):
    def __init__(self, record: int, what: str):
        super().__init__(f"record {record}: {what}")
        self.record = record


def _read_until_nl(buf: bytes, pos: int) -> tuple[bytes, int]:
    if pos >= len(buf):
        return b"", pos
    j = buf.find(b"\n", pos)
    end = len(buf) if j < 0 else j + 1
    return buf[pos:end], end


def _trim(line: bytes) -> bytes:
    end = len(line)
    while end and line[end - 1] in (10, 13):
        end -= 1
    return line[:end]


def parse_fastq(buf: bytes) -> list[tuple[bytes, bytes, bytes]]:
    """FastqReader::next until EOF: (id, sequence, quality) per record."""
    recs = []
    pos = 0
    while True:
        line, pos = _read_until_nl(buf, pos)
        if not line:
            return recs
        rid = _trim(line)
        line, pos = _read_until_nl(buf, pos)
        seq = _trim(line)
        sep, pos = _read_until_nl(buf, pos)
        if not sep:
            raise FastqError(len(recs), "unexpected EOF at '+' separator line")
        if sep[0] != ord("+"):
            raise FastqError(len(recs), "expected '+' separator line")
        line, pos = _read_until_nl(buf, pos)
        if not line:
            raise FastqError(len(recs), "unexpected EOF at quality line")
        qual = _trim(line)
        if len(qual) != len(seq):
            raise FastqError(len(recs), "sequence length != quality length")
        recs.append((rid, seq, qual))


def varint(v: int) -> bytes:
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def pack_qualities(q: bytes) -> bytes:
    out = bytearray()
    buf = 0
    nbits = 0
    for c in q:
        enc = min(max(c - 33, 0), 127)
        buf |= enc << nbits
        nbits += 7
        while nbits >= 8:
            out.append(buf & 0xFF)
            buf >>= 8
            nbits -= 8
    if nbits:
        out.append(buf & 0xFF)
    return bytes(out)


def const_lengths(recs) -> tuple[int, int]:
    if not recs:
        return 0, 0
    s0, q0 = len(recs[0][1]), len(recs[0][2])
    cs = s0 if all(len(r[1]) == s0 for r in recs) else 0
    cq = q0 if all(len(r[2]) == q0 for r in recs) else 0
    return cs, cq


def fastq_streams(buf: bytes):
    """(header stream, sequence stream, quality stream, records, const_seq_len,
    const_qual_len) of a FASTQ buffer; raises FastqError like the reader."""
    recs = parse_fastq(bytes(buf))
    cs, cq = const_lengths(recs)
    hdr, seq, qual = bytearray(), bytearray(), bytearray()
    for rid, s, q in recs:
        hdr += varint(len(rid))
        hdr += rid
        if cs == 0:
            seq += varint(len(s))
        seq += s
        if cq == 0:
            qual += varint(len(q))
        qual += pack_qualities(q)
    return bytes(hdr), bytes(seq), bytes(qual), len(recs), cs, cq
