"""Seeded synthetic block workloads with the shapes of qz's BSC streams.

The byte layouts follow qz's stream builder, so every block is what qz would
hand to the block sorter:

* sequences: bases concatenated with no length varints, because the reads have
  a constant length (compression/mod.rs:270-325, const_seq_len path at :297-299);
* qualities: lossless Phred values packed 7 bits each, LSB first, padded per
  read (compression/columnar.rs:104-134; 150 quals -> 132 bytes);
* headers: ``[varint(len)][id including '@']`` per read (mod.rs:291-292,
  varint at mod.rs:683-689);
* block cut: 25 MiB = 26,214,400 bytes (mod.rs:388-413, cli.rs:133).

No public dataset is read: the reference measured on ERR3239334, which is not
available here, so seeded synthetic reads of the same shape stand in for it.
"""
from __future__ import annotations

import math

import numpy as np

BLOCK_BYTES = 25 * 1024 * 1024  # qz's default bsc_block_size_mb = 25
READ_LEN = 150
QUAL_VALUES = np.array([2, 12, 23, 37], dtype=np.uint8)
_ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
_COMP = np.zeros(256, dtype=np.uint8)
for _a, _b in zip(b"ACGTN", b"TGCAN"):
    _COMP[_a] = _b


# --------------------------------------------------------------------------- genomes


def uniform_genome(length: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return _ACGT[rng.integers(0, 4, length)]


def repeat_genome(length: int, seed: int, cover: float = 0.20, max_run: int = 10_000) -> np.ndarray:
    """Uniform ACGT genome with tandem repeats (period 2-6, runs up to
    ``max_run`` bases) placed until they cover ``cover`` of the length."""
    rng = np.random.default_rng(seed)
    g = _ACGT[rng.integers(0, 4, length)]
    covered = 0
    target = int(cover * length)
    while covered < target:
        period = int(rng.integers(2, 7))
        run = int(rng.integers(period * 4, max_run + 1))
        start = int(rng.integers(0, length - run))
        unit = _ACGT[rng.integers(0, 4, period)]
        g[start:start + run] = np.resize(unit, run)
        covered += run
    return g


# --------------------------------------------------------------------------- reads


def sample_reads(genome: np.ndarray, nreads: int, seed: int, read_len: int = READ_LEN,
                 sub_rate: float = 1e-3, n_rate: float = 1e-4, chunk: int = 200_000) -> np.ndarray:
    """Reads sampled uniformly, 50% reverse complement, with uniform
    substitutions and Ns. Returns the concatenated sequence stream."""
    rng = np.random.default_rng(seed)
    out = np.empty(nreads * read_len, dtype=np.uint8)
    span = len(genome) - read_len + 1
    offs = np.arange(read_len, dtype=np.int64)
    for lo in range(0, nreads, chunk):
        m = min(chunk, nreads - lo)
        starts = rng.integers(0, span, m)
        reads = genome[starts[:, None] + offs[None, :]]
        rc = rng.random(m) < 0.5
        reads[rc] = _COMP[reads[rc][:, ::-1]]
        sub = rng.random((m, read_len)) < sub_rate
        if sub.any():
            cur = reads[sub]
            shift = rng.integers(1, 4, cur.shape[0])
            idx = (np.searchsorted(_ACGT, cur) + shift) % 4
            reads[sub] = np.where(np.isin(cur, _ACGT), _ACGT[idx], cur)
        nmask = rng.random((m, read_len)) < n_rate
        reads[nmask] = ord("N")
        out[lo * read_len:(lo + m) * read_len] = reads.reshape(-1)
    return out


def _quality_chunks(nreads: int, seed: int, read_len: int, chunk: int):
    """(first read, Phred values of up to `chunk` reads) from the quality model."""
    rng = np.random.default_rng(seed)
    stay = 0.95 - 0.15 * np.arange(read_len) / max(read_len - 1, 1)
    init_p = np.array([0.05, 0.10, 0.25, 0.60])
    for lo in range(0, nreads, chunk):
        m = min(chunk, nreads - lo)
        state = rng.choice(4, size=m, p=init_p)
        q = np.empty((m, read_len), dtype=np.uint8)
        for t in range(read_len):
            if t:
                move = rng.random(m) >= stay[t]
                step = rng.integers(1, 4, m)
                state = np.where(move, (state + step) % 4, state)
            q[:, t] = QUAL_VALUES[state]
        yield lo, q


def quality_values(nreads: int, seed: int, read_len: int = READ_LEN, chunk: int = 200_000) -> np.ndarray:
    """Phred values (reads x read_len) of the quality model below."""
    out = np.empty((nreads, read_len), dtype=np.uint8)
    for lo, q in _quality_chunks(nreads, seed, read_len, chunk):
        out[lo:lo + len(q)] = q
    return out


def quality_stream(nreads: int, seed: int, read_len: int = READ_LEN, chunk: int = 200_000) -> np.ndarray:
    """Phred values {2,12,23,37} from a per-read Markov chain whose
    stay-probability falls linearly from 0.95 to 0.80 along the read, packed
    7 bits per value LSB-first per read (columnar.rs:104-134)."""
    per_read = (read_len * 7 + 7) // 8
    out = np.empty(nreads * per_read, dtype=np.uint8)
    for lo, q in _quality_chunks(nreads, seed, read_len, chunk):
        m = len(q)
        bits = ((q[:, :, None] >> np.arange(7, dtype=np.uint8)) & 1).reshape(m, read_len * 7)
        pad = per_read * 8 - read_len * 7
        if pad:
            bits = np.concatenate([bits, np.zeros((m, pad), dtype=np.uint8)], axis=1)
        out[lo * per_read:(lo + m) * per_read] = np.packbits(bits, axis=1, bitorder="little").reshape(-1)
    return out


def _varint(v: int) -> bytes:
    b = bytearray()
    while v >= 0x80:
        b.append((v & 0x7F) | 0x80)
        v >>= 7
    b.append(v)
    return bytes(b)


def header_ids(nreads: int, seed: int) -> list[bytes]:
    """Illumina-style ids '@SIM:1:FC01:<lane>:<tile>:<x>:<y> 1:N:0:<8-mer>',
    reads laid out lane by lane and tile by tile with x and y increasing within
    each tile; one sample index per lane with rare single-base errors."""
    rng = np.random.default_rng(seed)
    lanes, tiles = 4, 2624 - 1101 + 1
    cells = lanes * tiles
    cell_of = np.sort(rng.integers(0, cells, nreads))
    counts = np.bincount(cell_of, minlength=cells)
    xs = np.empty(nreads, dtype=np.int64)
    ys = np.empty(nreads, dtype=np.int64)
    pos = 0
    for c in range(cells):
        k = int(counts[c])
        if k:
            xs[pos:pos + k] = np.sort(rng.integers(1, 32001, k))
            ys[pos:pos + k] = np.sort(rng.integers(1, 32001, k))
            pos += k
    lane_idx = [bytes(_ACGT[rng.integers(0, 4, 8)]) for _ in range(lanes)]
    err = rng.random(nreads) < 0.005
    err_pos = rng.integers(0, 8, nreads)
    err_base = rng.integers(0, 4, nreads)
    ids = []
    for r in range(nreads):
        c = int(cell_of[r])
        lane, tile = c // tiles, 1101 + c % tiles
        idx = lane_idx[lane]
        if err[r]:
            b = bytearray(idx)
            b[err_pos[r]] = b"ACGT"[err_base[r]]
            idx = bytes(b)
        ids.append(b"@SIM:1:FC01:%d:%d:%d:%d 1:N:0:%s" % (lane + 1, tile, xs[r], ys[r], idx))
    return ids


def header_stream(nreads: int, seed: int) -> np.ndarray:
    """header_ids laid out as qz's header stream ``[varint(len)][id]``
    (mod.rs:291-292)."""
    parts = []
    for s in header_ids(nreads, seed):
        parts.append(_varint(len(s)))
        parts.append(s)
    return np.frombuffer(b"".join(parts), dtype=np.uint8).copy()


def fastq_text(ids: list[bytes], seqs: np.ndarray, quals: np.ndarray, chunk: int = 100_000) -> np.ndarray:
    """FASTQ text ('\n' line ends) of reads with one length: id line, bases,
    '+', Phred+33 qualities."""
    n, L = seqs.shape
    id_lens = np.fromiter((len(i) for i in ids), dtype=np.int64, count=n)
    rec_len = id_lens + 2 * L + 5  # id, bases, "+", qualities, each with its newline
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(rec_len, out=off[1:])
    out = np.empty(int(off[-1]), dtype=np.uint8)
    ar = np.arange(L, dtype=np.int64)
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        ic = np.frombuffer(b"".join(ids[lo:hi]), dtype=np.uint8)
        il = id_lens[lo:hi]
        starts = off[lo:hi]
        ioff = np.zeros(hi - lo, dtype=np.int64)
        np.cumsum(il[:-1], out=ioff[1:])
        out[np.repeat(starts - ioff, il) + np.arange(ic.size)] = ic
        nl = starts + il
        out[nl] = 10
        sq = nl + 1
        out[sq[:, None] + ar] = seqs[lo:hi]
        out[sq + L] = 10
        out[sq + L + 1] = ord("+")
        out[sq + L + 2] = 10
        qs = sq + L + 3
        out[qs[:, None] + ar] = quals[lo:hi] + 33
        out[qs + L] = 10
    return out


def chunk_fastq(nreads: int = 2_500_000) -> np.ndarray:
    """The FASTQ text whose three qz streams are chunk_blocks' streams (same
    genome, reads, qualities and ids; seeds 1-4)."""
    g = uniform_genome(5_000_000, seed=1)
    seq = sample_reads(g, nreads, seed=2).reshape(nreads, READ_LEN)
    qual = quality_values(nreads, seed=3)
    return fastq_text(header_ids(nreads, seed=4), seq, qual)


def cut_blocks(stream: np.ndarray, block_bytes: int = BLOCK_BYTES) -> list[np.ndarray]:
    """compress_stream_to_bsc_blocks' cut (mod.rs:388-413): fixed-size chunks."""
    return [stream[i:i + block_bytes] for i in range(0, len(stream), block_bytes)]


# --------------------------------------------------------------------------- configs


def plain_block(nreads: int = 166_666) -> np.ndarray:
    """One 24,999,900-byte sequence block: 166,666 x 150 bp reads from a
    seeded 5 Mbp genome (seed 1), reads seed 2."""
    g = uniform_genome(5_000_000, seed=1)
    return sample_reads(g, nreads, seed=2)


def chunk_blocks(nreads: int = 2_500_000) -> list[tuple[str, np.ndarray]]:
    """One qz chunk split into its three streams and cut into 25 MiB blocks:
    ~15 sequence, 13 quality and 5 header blocks for 2.5M reads."""
    g = uniform_genome(5_000_000, seed=1)
    seq = sample_reads(g, nreads, seed=2)
    qual = quality_stream(nreads, seed=3)
    hdr = header_stream(nreads, seed=4)
    out = []
    for kind, s in (("seq", seq), ("qual", qual), ("hdr", hdr)):
        out.extend((kind, b) for b in cut_blocks(s))
    return out


def ultra_block(nbytes: int = 750 * 1024 * 1024, seed: int = 8) -> np.ndarray:
    """One ultra-mode sequence block (qz's reorder levels use BSC blocks up to
    750 MiB, ultra.rs:44-55): 150 bp reads from a 50 Mbp genome (seed 8),
    truncated to `nbytes`."""
    g = uniform_genome(50_000_000, seed=seed)
    reads = nbytes // READ_LEN + 1
    return sample_reads(g, reads, seed=seed + 1)[:nbytes]


def _source_streams(max_len: int, seed: int) -> dict[str, np.ndarray]:
    reads = max_len // READ_LEN + 1
    g = uniform_genome(5_000_000, seed=1)
    return {
        "dna": sample_reads(g, reads, seed=seed),
        "qual": quality_stream(max_len // 132 + 1, seed=seed + 1),
        "hdr": header_stream(max_len // 40 + 1, seed=seed + 2),
    }


def uneven_blocks(count: int = 256, lo: int = 1024, hi: int = BLOCK_BYTES, seed: int = 5,
                  max_source: int | None = None) -> list[tuple[str, np.ndarray]]:
    """Uneven-size batch: sizes log-uniform on [lo, hi], types 50% DNA, 30%
    quality, 20% header, each a contiguous slice of a generated stream."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    kinds = rng.choice(["dna", "qual", "hdr"], size=count, p=[0.5, 0.3, 0.2])
    src = _source_streams(int(max_source or sizes.max()), seed=seed * 100)
    out = []
    for s, k in zip(sizes, kinds):
        stream = src[str(k)]
        s = int(min(s, len(stream)))
        off = int(rng.integers(0, len(stream) - s + 1))
        out.append((str(k), stream[off:off + s]))
    return out


def serving_requests(count: int, rate_per_s: float, seed: int = 6, lo: int = 65_536,
                     hi: int = BLOCK_BYTES, max_source: int | None = None):
    """Poisson arrivals; sizes log-uniform on [lo, hi] with the uneven-batch
    type mix; 70% forward (compress) and 30% inverse (decompress) requests.
    Returns a list of (arrival_s, op, kind, block)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, count)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    kinds = rng.choice(["dna", "qual", "hdr"], size=count, p=[0.5, 0.3, 0.2])
    ops = np.where(rng.random(count) < 0.7, "fwd", "inv")
    src = _source_streams(int(max_source or sizes.max()), seed=seed * 100)
    out = []
    for a, s, k, op in zip(arrivals, sizes, kinds, ops):
        stream = src[str(k)]
        s = int(min(s, len(stream)))
        off = int(rng.integers(0, len(stream) - s + 1))
        out.append((float(a), str(op), str(k), stream[off:off + s]))
    return out


def repeat_blocks(reads: int = 120_000) -> list[tuple[str, np.ndarray]]:
    """Worst case for deep suffix comparisons: 250 bp reads at 30x over a
    seeded 1 Mbp genome with 20% tandem repeats (two blocks), one block of a
    single repeated byte and one block of 'ACG' repeats."""
    g = repeat_genome(1_000_000, seed=7)
    seq = sample_reads(g, reads, seed=8, read_len=250)
    out = [("repeat", b) for b in cut_blocks(seq)]
    out.append(("single", np.full(BLOCK_BYTES, ord("A"), dtype=np.uint8)))
    out.append(("period3", np.resize(np.frombuffer(b"ACG", dtype=np.uint8), BLOCK_BYTES)))
    return out
