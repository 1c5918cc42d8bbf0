"""GPU parity at the workloads' own sizes: every block of each workload the
benchmark runs, forward BWT through the C ABI against the C oracle (SA-IS,
threaded one block per host core), bit-exact (bytes and primary indexes),
then the GPU inverse of the GPU output back to the input.

The call whose output must match is libbsc's BWT stage inside bsc_compress
(crates/qz-lib/src/compression/bsc.rs:172-183); the inverse is the one inside
bsc_decompress (bsc.rs:421-433).

Workloads (seeded synthetic stand-ins of the reference's read sets):
  * one 24,999,900-byte sequence block (166,666 x 150 bp reads, 5 Mbp genome);
  * one qz chunk: 2.5M reads cut into 33 blocks of 25 MiB (818 MB);
  * 64 of the 256 uneven blocks (1 KB-25 MiB, DNA / quality / header mix),
    the largest one included;
  * served requests (64 KB-25 MiB) through the serving loop;
  * repeat-rich reads (26,214,400 + 3,785,600 bytes), a 26,214,400-byte block
    of one repeated byte and one of 'ACG' repeats (the deepest doubling);
  * one 750 MiB ultra-mode block.
"""
import os

import numpy as np
import pytest

from qz_gb300 import bwt, synth

pytestmark = pytest.mark.gpu
CORES = os.cpu_count() or 1


@pytest.fixture(scope="module")
def gpu():
    bwt.init()
    return True


def check_batch(oracle, blocks, storage_bytes=None):
    """GPU batch forward vs the oracle, block by block; GPU inverse back to
    the input.  Returns the number of doubling rounds the GPU needed."""
    total = storage_bytes or sum(len(b) for b in blocks)
    with bwt.Storage(total, len(blocks)) as st:
        us, idx = st.encode_batch(blocks)
        rounds = st.stats()["rounds"]
        ous, oidx = oracle.bwt_encode_batch(blocks, threads=CORES)
        bad = [i for i, (u, ou, p, op) in enumerate(zip(us, ous, idx, oidx)) if p != op or not np.array_equal(u, ou)]
        assert not bad, f"blocks differing from the oracle: {bad[:10]} (sizes {[len(blocks[i]) for i in bad[:10]]})"
        back = st.decode_batch(us, idx)
        bad = [i for i, (x, y) in enumerate(zip(back, blocks)) if not np.array_equal(x, y)]
        assert not bad, f"inverse differs from the input in blocks {bad[:10]}"
    return rounds


def test_plain_block_25mb(gpu, oracle):
    t = synth.plain_block()
    assert len(t) == 24_999_900
    check_batch(oracle, [t])
    # the single-block drop-in (libbsc's in-place call shape) on the same block
    u, idx = bwt.bwt_encode(t)
    ou, oidx = oracle.bwt_encode(t)
    assert idx == oidx and np.array_equal(u, ou)
    assert np.array_equal(bwt.bwt_decode(u, idx), t)


def test_chunk_all_33_blocks(gpu, oracle):
    blocks = [b for _, b in synth.chunk_blocks()]
    assert len(blocks) == 33 and sum(len(b) for b in blocks) == 818_264_088
    check_batch(oracle, blocks)


def test_uneven_batch_slice_with_largest_block(gpu, oracle):
    blocks = [b for _, b in synth.uneven_blocks(256)]
    order = np.argsort([len(b) for b in blocks])
    pick = sorted(set([int(order[-1])] + [int(i) for i in order[::4][:63]]))
    sl = [blocks[i] for i in pick]
    assert len(sl) == 64 and max(len(b) for b in sl) == max(len(b) for b in blocks)
    check_batch(oracle, sl)


def test_served_requests_match_oracle(gpu, oracle):
    reqs = synth.serving_requests(24, rate_per_s=1.0, seed=6)
    fwd = [b for _, op, _, b in reqs]
    ous, oidx = oracle.bwt_encode_batch(fwd, threads=CORES)
    with bwt.Server(hbm_budget=0, max_slots=3, slot_bytes=64 << 20, slot_blocks=64) as srv:
        tickets = [srv.submit_forward(b) for b in fwd]
        got = [srv.wait(t) for t in tickets]
        for r, ou, oi in zip(got, ous, oidx):
            assert r["index"] == oi and np.array_equal(r["out"], ou)
        inv = [srv.submit_inverse(ou, oi) for ou, oi in zip(ous, oidx)]
        for t, b in zip(inv, fwd):
            assert np.array_equal(srv.wait(t)["out"], b)


def test_repeat_rich_reads(gpu, oracle):
    blocks = [b for k, b in synth.repeat_blocks() if k == "repeat"]
    assert [len(b) for b in blocks] == [26_214_400, 3_785_600]
    check_batch(oracle, blocks)


@pytest.mark.parametrize("kind", ["single", "period3"])
def test_deepest_doubling_blocks(gpu, oracle, kind):
    t = [b for k, b in synth.repeat_blocks(reads=1) if k == kind][0]
    assert len(t) == 26_214_400
    rounds = check_batch(oracle, [t])
    if kind == "period3":
        assert rounds >= 20  # about log2(n) doubling rounds


def test_ultra_block_750mib(gpu, oracle):
    t = synth.ultra_block()
    assert len(t) == 750 << 20
    check_batch(oracle, [t])
