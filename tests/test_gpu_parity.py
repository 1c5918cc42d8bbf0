"""GPU parity: the sm_103a forward / inverse BWT through the C ABI against the
CPU oracle, bit-exact (integer and byte work: no tolerance).

Test names follow the reference's BSC unit tests (bsc.rs:438-499) where they
cover the same case, at block level.
"""
import json
import os

import numpy as np
import pytest

from qz_gb300 import bwt, native, synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bwt_vectors.json")


@pytest.fixture(scope="module")
def gpu():
    bwt.init()
    return True


def _check_block(oracle, t):
    t = np.ascontiguousarray(t, dtype=np.uint8)
    u, idx = bwt.bwt_encode(t)
    if len(t):
        ou, oidx = oracle.bwt_encode(t)
        assert idx == oidx
        assert (u == ou).all()
    else:
        assert idx == 0 and len(u) == 0
    back = bwt.bwt_decode(u, idx)
    assert (back == t).all()


@pytest.mark.parametrize("vec", json.load(open(GOLDEN))["vectors"], ids=lambda v: v["name"])
def test_golden_vectors(gpu, vec):
    t = bytes.fromhex(vec["input"])
    u, idx, aux = bwt.bwt_encode(t, with_aux=True)
    assert bytes(u) == bytes.fromhex(vec["bwt"])
    assert idx == vec["index"]
    assert bytes(bwt.bwt_decode(u, idx)) == t


def test_roundtrip_simple(gpu, oracle):
    _check_block(oracle, np.frombuffer(b"ACGTACGTACGTACGTACGTACGTACGTACGT", np.uint8))


def test_roundtrip_genomic(gpu, oracle):
    g = synth.uniform_genome(50_000, seed=21)
    _check_block(oracle, synth.sample_reads(g, 2000, seed=22))


def test_roundtrip_quality(gpu, oracle):
    _check_block(oracle, synth.quality_stream(3000, seed=23))


def test_roundtrip_headers(gpu, oracle):
    _check_block(oracle, synth.header_stream(5000, seed=24))


def test_empty_data(gpu):
    u, idx = bwt.bwt_encode(b"")
    assert len(u) == 0 and idx == 0
    assert len(bwt.bwt_decode(b"", 0)) == 0


@pytest.mark.parametrize("n", [1, 2, 3, 15, 16, 17, 31, 33, 255, 4095, 4096, 4097, 8193, 70_000])
@pytest.mark.parametrize("sigma", [1, 2, 5, 256])
def test_sizes_and_alphabets(gpu, oracle, n, sigma):
    rng = np.random.default_rng(n * 1000 + sigma)
    _check_block(oracle, rng.integers(0, sigma, n).astype(np.uint8))


@pytest.mark.parametrize("kind", ["single", "period2", "period3", "period7", "runs"])
def test_repetitive(gpu, oracle, kind):
    n = 200_000
    if kind == "single":
        t = np.full(n, 65, np.uint8)
    elif kind == "runs":
        rng = np.random.default_rng(5)
        t = np.repeat(rng.integers(0, 3, n // 1000).astype(np.uint8), 1000)
    else:
        p = int(kind[6:])
        t = np.resize(np.frombuffer(b"ACGTNQZ"[:p], np.uint8), n)
    _check_block(oracle, t)


def test_tandem_repeat_reads(gpu, oracle):
    g = synth.repeat_genome(100_000, seed=31)
    _check_block(oracle, synth.sample_reads(g, 3000, seed=32, read_len=250))


def test_aux_indexes_match_oracle(gpu, oracle):
    t = synth.sample_reads(synth.uniform_genome(20_000, seed=41), 400, seed=42)
    u, idx, aux = bwt.bwt_encode(t, with_aux=True)
    r = bwt.aux_rate(len(t))
    ou, oidx, oaux = oracle.bwt_encode(t, aux_rate=r)
    assert idx == oidx and list(aux) == list(oaux[1:])


def test_batch_uneven_matches_single(gpu, oracle):
    rng = np.random.default_rng(77)
    blocks = []
    for i in range(40):
        n = int(np.exp(rng.uniform(0, np.log(300_000))))
        kind = i % 4
        if kind == 0:
            blocks.append(rng.integers(0, 4, n).astype(np.uint8) + 65)
        elif kind == 1:
            blocks.append(rng.integers(0, 256, n).astype(np.uint8))
        elif kind == 2:
            blocks.append(np.full(n, 7, np.uint8))
        else:
            blocks.append(np.resize(np.frombuffer(b"ACG", np.uint8), n))
    blocks.insert(3, np.zeros(0, np.uint8))
    blocks.insert(9, np.array([42], np.uint8))
    total = sum(len(b) for b in blocks)
    with bwt.Storage(total, len(blocks)) as st:
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        for b, u, i, ou, oi in zip(blocks, us, idx, ous, oidx):
            assert len(u) == len(b)
            if len(b):
                assert i == oi
                assert (u == ou).all()
        back = st.decode_batch(us, idx)
        assert all((x == y).all() for x, y in zip(back, blocks))


def test_decode_rejects_corrupt_index(gpu):
    t = synth.sample_reads(synth.uniform_genome(5000, seed=51), 50, seed=52)
    u, idx = bwt.bwt_encode(t)
    for bad in (0, len(t) + 1):
        with pytest.raises(native.QzGpuError) as e:
            bwt.bwt_decode(u, bad)
        assert e.value.code == native.QZGPU_DATA_CORRUPT


def test_decode_wrong_index_does_not_hang(gpu):
    # A wrong but in-range index yields some permutation or a corrupt-cycle
    # error; either way the call returns.
    t = synth.sample_reads(synth.uniform_genome(5000, seed=53), 50, seed=54)
    u, idx = bwt.bwt_encode(t)
    wrong = idx % len(t) + 1
    try:
        out = bwt.bwt_decode(u, wrong)
        assert len(out) == len(t)
    except native.QzGpuError as e:
        assert e.code == native.QZGPU_DATA_CORRUPT


@pytest.mark.parametrize("mode,early", [(1, 0), (1, 1), (2, 0)])
def test_lookback_wait_runs_out_without_fault(gpu, oracle, mode, early):
    # Failure detection: in the test mode one tile never publishes its
    # look-back status (mode 1: a tile of every large group in the radix sort;
    # mode 2: the second tile of every one-pass split), so the tiles
    # behind it give up after a short bounded wait; the call returns
    # QZGPU_TIMEOUT (no fault, no hang) and the same storage sorts correctly
    # once the mode is off.  `early`: the radix tiles publish their counts
    # before their ranking.
    rng = np.random.default_rng(5)
    blocks = [rng.integers(0, 256, 1 << 20).astype(np.uint8)]  # one 2^20-slot group at the start
    with bwt.Storage(len(blocks[0]), 1) as st:
        st.set_param("early_counts", early)
        st.set_param("split_lookback", 1 if mode == 2 else 0)
        st.set_param("lookback_test", mode)
        with pytest.raises(native.QzGpuError) as e:
            st.encode_batch(blocks)
        assert e.value.code == native.QZGPU_TIMEOUT
        st.set_param("lookback_test", 0)
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert (us[0] == ous[0]).all()
        with pytest.raises(native.QzGpuError):
            st.set_param("lookback_test", 3)


@pytest.mark.parametrize("params", [
    {"medium_max": 64, "big_ctas_per_sm": 2, "ruler_stride_log2": 3, "round_pipeline": 1},
    {"split_lookback": 1, "rank_mode": 1, "early_counts": 1},
    {"split_lookback": 1, "round_pipeline": 1, "medium_max": 128, "rank_mode": 2},
    {"medium_max": 512, "big_ctas_per_sm": 4, "fwd_sub_bytes": 1 << 20, "big_tile": 2048, "rank_mode": 1},
    {"medium_max": 128, "tile_ctas_per_sm": 1, "ruler_stride_log2": 7, "fwd_sub_bytes": 1 << 20,
     "inv_sub_bytes": 1 << 20, "big_tile": 8192, "radix_first_bits": 8, "round_pipeline": 1},
    {"medium_max": 256, "big_ctas_per_sm": 1, "ruler_stride_log2": 4, "radix_first_bits": 9, "early_counts": 1},
    {"rank_mode": 2, "early_counts": 1, "big_tile": 8192, "pass0_bulk": 0},
    {"rank_mode": 0, "early_counts": 0, "medium_max": 64, "pass0_bulk": 0},
    {"pass0_bulk": 1, "big_tile": 2048, "radix_first_bits": 8},
    {"pass0_bulk": 1, "fwd_sub_bytes": 1 << 20, "round_pipeline": 1},
    {"ruler_stride_log2": 12, "round_pipeline": 1, "big_ctas_per_sm": 4},
])
def test_tuned_knobs_keep_results(gpu, oracle, params):
    rng = np.random.default_rng(99)
    blocks = [synth.sample_reads(synth.uniform_genome(30_000, seed=71), 1500, seed=72),
              synth.quality_stream(4000, seed=73), synth.header_stream(6000, seed=74),
              np.resize(np.frombuffer(b"ACG", np.uint8), 90_000), rng.integers(0, 256, 5000).astype(np.uint8)]
    with bwt.Storage(sum(len(b) for b in blocks), len(blocks)) as st:
        for k, v in params.items():
            st.set_param(k, v)
            assert st.get_param(k) == v
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))
        back = st.decode_batch(us, idx)
        assert all((x == y).all() for x, y in zip(back, blocks))
        with pytest.raises(native.QzGpuError):
            st.set_param("medium_max", 100)


def test_profile_only_times_one_kernel(gpu):
    blocks = [synth.sample_reads(synth.uniform_genome(20_000, seed=81), 200, seed=82)]
    with bwt.Storage(len(blocks[0]), 1) as st:
        st.profile(True, only="k_extract")
        st.encode_batch(blocks)
        names = {r["name"] for r in st.profile_read()}
        assert names == {"k_extract"}
        st.profile(True)
        st.encode_batch(blocks)
        assert len(st.profile_read()) > 3
        st.profile(False)


def _big_blocks():
    g = synth.uniform_genome(400_000, seed=91)
    return [synth.sample_reads(g, 20_000, seed=92 + i) for i in range(3)]  # 3 x 3 MB


def test_batch_fresh_outputs_above_touch_threshold(gpu, oracle):
    # more than 8 MiB of host output: the engine touches the output pages on a
    # host thread while the device works
    blocks = _big_blocks()
    with bwt.Storage(sum(len(b) for b in blocks), len(blocks)) as st:
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))
        back = st.decode_batch(us, idx)
        assert all((x == y).all() for x, y in zip(back, blocks))


@pytest.mark.parametrize("pinned", ["all", "some"])
def test_batch_pinned_outputs_above_touch_threshold(gpu, oracle, pinned):
    # page-locked outputs are resident: the engine skips touching them (all
    # pinned); one pageable output among them brings the touching back
    import torch
    blocks = _big_blocks()

    def out(n, i):
        if pinned == "some" and i == 1:
            return np.empty(n, np.uint8)
        return torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy()

    with bwt.Storage(sum(len(b) for b in blocks), len(blocks)) as st:
        us, idx = st.encode_batch(blocks, out=[out(len(b), i) for i, b in enumerate(blocks)])
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))
        back = st.decode_batch(us, idx, out=[out(len(b), i) for i, b in enumerate(blocks)])
        assert all((x == y).all() for x, y in zip(back, blocks))


def test_batch_in_place_above_touch_threshold(gpu, oracle):
    import ctypes
    blocks = _big_blocks()
    work = [b.copy() for b in blocks]
    nb = len(work)
    sizes = np.array([len(b) for b in work], dtype=np.int32)
    idx = np.zeros(nb, dtype=np.int32)
    u8p = ctypes.POINTER(ctypes.c_uint8)
    ptrs = (u8p * nb)(*[b.ctypes.data_as(u8p) for b in work])
    with bwt.Storage(int(sizes.sum()), nb) as st:
        lib = native.load()
        i32p = ctypes.POINTER(ctypes.c_int32)
        rc = lib.qzgpu_bwt_encode_batch(st._h, nb, ptrs, ptrs, sizes.ctypes.data_as(i32p), idx.ctypes.data_as(i32p), 0)
        assert rc == 0
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert list(idx) == list(oidx)
        assert all((w == ou).all() for w, ou in zip(work, ous))
        rc = lib.qzgpu_bwt_decode_batch(st._h, nb, ptrs, ptrs, sizes.ctypes.data_as(i32p), idx.ctypes.data_as(i32p), 0)
        assert rc == 0
        assert all((w == b).all() for w, b in zip(work, blocks))


def test_batch_out_buffers_reused(gpu):
    blocks = [synth.quality_stream(2000, seed=95), synth.header_stream(3000, seed=96), np.zeros(0, np.uint8)]
    with bwt.Storage(sum(len(b) for b in blocks), len(blocks)) as st:
        us0, idx0 = st.encode_batch(blocks)
        outs = [np.empty(len(b), np.uint8) for b in blocks]
        back = [np.empty(len(b), np.uint8) for b in blocks]
        for _ in range(2):
            us, idx = st.encode_batch(blocks, out=outs)
            assert idx[:2] == idx0[:2]
            assert all((u == v).all() for u, v in zip(us, us0))
            assert all(u.base is o or u is o or np.shares_memory(u, o) for u, o in zip(us[:2], outs[:2]))
            st.decode_batch(us, idx, out=back)
            assert all((x == y).all() for x, y in zip(back, blocks))
        with pytest.raises(native.QzGpuError):
            st.encode_batch(blocks, out=outs[:2])


@pytest.mark.parametrize("kind", ["header", "quality"])
def test_large_repetitive_blocks(gpu, oracle, kind):
    # multi-megabyte header / quality blocks: large groups over several rounds,
    # radix passes skipped where a group's digit is constant
    t = synth.header_stream(120_000, seed=97) if kind == "header" else synth.quality_stream(40_000, seed=98)
    _check_block(oracle, t)
    with bwt.Storage(2 * len(t), 2) as st:
        us, idx = st.encode_batch([t, t[: len(t) // 2]])
        ous, oidx = oracle.bwt_encode_batch([t, t[: len(t) // 2]])
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))


def test_block_above_lane_size(gpu, oracle):
    # an 80 MB block is larger than a lane's 64 MiB sub-batch: it runs alone on
    # the full-capacity lane, next to small blocks on the others
    g = synth.uniform_genome(2_000_000, seed=99)
    big = synth.sample_reads(g, 80_000_000 // 150, seed=100)
    small = [synth.quality_stream(3000, seed=101), synth.header_stream(4000, seed=102)]
    blocks = [small[0], big, small[1]]
    with bwt.Storage(sum(len(b) for b in blocks), len(blocks)) as st:
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))
        back = st.decode_batch(us, idx)
        assert all((x == y).all() for x, y in zip(back, blocks))


def test_lanes_take_largest_sub_batches_first(gpu, oracle):
    # a three-lane storage (capacity above 64 MiB) with 1 MiB sub-batches:
    # twelve uneven blocks (11 MB of fresh host output, so the output pages are
    # touched on a host thread in the order the lanes work) are cut into
    # sub-batches that the lanes take largest first; every block must come
    # back in its own place
    rng = np.random.default_rng(7)
    sizes = [int(x) for x in rng.integers(1000, 1_800_000, 12)]
    g = synth.uniform_genome(300_000, seed=8)
    blocks = [synth.sample_reads(g, s // 150 + 1, seed=9 + i)[:s] for i, s in enumerate(sizes)]
    with bwt.Storage(65 << 20, 16) as st:
        assert st.get_param("lanes") == 3
        st.set_param("fwd_sub_bytes", 1 << 20)
        st.set_param("inv_sub_bytes", 1 << 20)
        us, idx = st.encode_batch(blocks)
        ous, oidx = oracle.bwt_encode_batch(blocks)
        assert idx == list(oidx)
        assert all((u == ou).all() for u, ou in zip(us, ous))
        back = st.decode_batch(us, idx)
        assert all((x == y).all() for x, y in zip(back, blocks))


def test_ultra_block_round_trip(gpu):
    # a 300 MiB block (qz's reorder levels use blocks up to 750 MiB): the
    # inverse of the forward is the input (size-independent property; the
    # oracle parity of the same path is checked at 80 MB above)
    t = synth.ultra_block(300 << 20)
    with bwt.Storage(len(t), 1) as st:
        (u,), (idx,) = st.encode_batch([t])
        assert 1 <= idx <= len(t)
        assert np.bincount(u, minlength=256).tolist() == np.bincount(t, minlength=256).tolist()
        (back,) = st.decode_batch([u], [idx])
        assert (back == t).all()


@pytest.mark.parametrize("cap,blocks", [(1 << 20, 1), (25 << 20, 4), (200 << 20, 64)])
def test_storage_bytes_match_allocation(gpu, cap, blocks):
    # serving admission and qz's VRAM check (check_cuda_vram, bsc.rs:50-82)
    # rely on qzgpu_storage_bytes predicting what a storage takes from HBM
    torch = pytest.importorskip("torch")
    with bwt.Storage(1 << 20, 1) as warm:  # module loading and context set-up happen before measuring
        warm.encode_batch([np.frombuffer(b"warm-up block", np.uint8)])
    torch.cuda.synchronize()
    want = bwt.Storage.device_bytes(cap, blocks)
    free0, _ = torch.cuda.mem_get_info()
    st = bwt.Storage(cap, blocks)
    try:
        free1, _ = torch.cuda.mem_get_info()
        taken = free0 - free1
        lanes = st.get_param("lanes")
        # each lane is one cudaMalloc, rounded up to the driver's 2 MiB pages
        assert want <= taken <= want + lanes * (2 << 20) + (4 << 20), (want, taken)
    finally:
        st.close()
