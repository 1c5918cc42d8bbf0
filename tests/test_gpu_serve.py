"""Serving form: concurrent mixed forward / inverse requests batched onto
resident slots give, request by request, the same result as the request run
alone (bit-exact); a request that fails fails alone; slots are admitted by the
free HBM read at admission time."""
import threading

import numpy as np
import pytest

from qz_gb300 import bwt, native, synth

pytestmark = pytest.mark.gpu


def _requests(seed=90, count=60):
    rng = np.random.default_rng(seed)
    g = synth.uniform_genome(400_000, seed=91)
    dna = synth.sample_reads(g, 20_000, seed=92)
    qual = synth.quality_stream(20_000, seed=93)
    hdr = synth.header_stream(20_000, seed=94)
    src = [dna, qual, hdr]
    reqs = []
    for i in range(count):
        s = src[int(rng.integers(0, 3))]
        n = int(np.exp(rng.uniform(np.log(2), np.log(600_000))))
        off = int(rng.integers(0, len(s) - n))
        reqs.append(s[off:off + n].copy())
    reqs.insert(5, np.zeros(0, np.uint8))
    reqs.insert(9, np.array([7], np.uint8))
    return reqs


def test_served_results_equal_alone_results():
    bwt.init()
    blocks = _requests()
    alone = [bwt.bwt_encode(b) for b in blocks]
    with bwt.Server(hbm_budget=16 << 30, max_slots=3, slot_bytes=2 << 20, slot_blocks=64) as srv:
        assert srv.slots == 1  # more are admitted under load
        results = {}

        def client(idx):
            tickets = []
            for i in idx:
                if i % 3 == 2 and len(blocks[i]) > 0:
                    u, p = alone[i]
                    tickets.append((i, "inv", srv.submit_inverse(u, p)))
                else:
                    tickets.append((i, "fwd", srv.submit_forward(blocks[i])))
            for i, kind, t in tickets:
                results[(i, kind)] = srv.wait(t)

        threads = [threading.Thread(target=client, args=(list(range(k, len(blocks), 4)),)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        stats = srv.stats()
    assert len(results) == len(blocks)
    for (i, kind), r in results.items():
        if kind == "fwd":
            u, p = alone[i]
            assert r["index"] == p
            assert np.array_equal(r["out"], u)
        else:
            assert np.array_equal(r["out"], blocks[i])
        assert r["latency_ms"] >= r["queue_ms"] >= 0
    assert stats["completed"] == len(blocks)
    assert stats["batches"] < len(blocks)  # requests were batched


def test_served_rejects_oversize_and_bad_index():
    bwt.init()
    with bwt.Server(hbm_budget=8 << 30, max_slots=1, slot_bytes=1 << 20, slot_blocks=8) as srv:
        with pytest.raises(native.QzGpuError):
            srv.submit_forward(np.zeros((1 << 20) + 1, np.uint8))
        with pytest.raises(native.QzGpuError) as e:
            srv.submit_inverse(np.frombuffer(b"ACGT", np.uint8), 9)
        assert e.value.code == native.QZGPU_DATA_CORRUPT


def _bad_inverse(oracle, n=50_000, seed=7):
    """A (U, index) pair that is not the BWT of anything: its LF mapping has
    more than one cycle, which the oracle rejects too."""
    rng = np.random.default_rng(seed)
    while True:
        u = rng.integers(65, 69, n).astype(np.uint8)
        idx = int(rng.integers(1, n + 1))
        try:
            oracle.bwt_decode(u, idx)
        except ValueError:
            return u, idx


def test_one_corrupt_inverse_fails_alone(oracle):
    # qz turns a failed bsc_decompress into an error for that call only
    # (bsc.rs:411-433); a served batch must not fail its other requests
    bwt.init()
    g = synth.uniform_genome(300_000, seed=95)
    good = [synth.sample_reads(g, 400 + 37 * i, seed=96 + i) for i in range(12)]
    enc = [bwt.bwt_encode(b) for b in good]
    bad_u, bad_idx = _bad_inverse(oracle)
    first_block = synth.sample_reads(g, 400_000, seed=94)  # 60 MB: keeps the slot busy for a while
    with bwt.Server(hbm_budget=16 << 30, max_slots=1, slot_bytes=64 << 20, slot_blocks=64) as srv:
        # one slot: every request that waits while the first batch runs goes
        # into one later batch with the corrupt request in its middle
        first = srv.submit_forward(first_block)
        tickets = [srv.submit_inverse(u, p) for u, p in enc[:6]]
        bad = srv.submit_inverse(bad_u, bad_idx)
        tickets += [srv.submit_inverse(u, p) for u, p in enc[6:]]
        assert srv.wait(first)["index"] >= 1
        with pytest.raises(native.QzGpuError) as e:
            srv.wait(bad)
        assert e.value.code == native.QZGPU_DATA_CORRUPT
        for t, b in zip(tickets, good):
            assert np.array_equal(srv.wait(t)["out"], b)
        stats = srv.stats()
    # the inverse requests queued behind the forward one: they ran in at most
    # two batches, so the corrupt request shared its batch
    assert stats["batches"] <= 3 and stats["max_batch"] >= 7


def test_wait_collects_a_ticket_once():
    bwt.init()
    with bwt.Server(hbm_budget=8 << 30, max_slots=1, slot_bytes=1 << 20, slot_blocks=8) as srv:
        t = srv.submit_forward(synth.quality_stream(500, seed=3))
        assert srv.wait(t) is not None
        with pytest.raises(native.QzGpuError) as e:
            srv.wait(t)
        assert e.value.code == native.QZGPU_BAD_PARAMETER


def _load(srv, blocks, rounds=3):
    for _ in range(rounds):
        ts = [srv.submit_forward(b) for b in blocks]
        for t in ts:
            srv.wait(t)


def test_slots_admitted_by_budget_and_free_hbm():
    torch = pytest.importorskip("torch")
    bwt.init()
    slot_bytes = 2 << 20
    per = bwt.Storage.device_bytes(slot_bytes, 16)
    g = synth.uniform_genome(200_000, seed=5)
    blocks = [synth.sample_reads(g, 10_000, seed=6 + i) for i in range(24)]  # 1.5 MB each
    # a budget of one and a half slots: never a second slot
    with bwt.Server(hbm_budget=per * 3 // 2, max_slots=4, slot_bytes=slot_bytes, slot_blocks=16) as srv:
        _load(srv, blocks)
        st = srv.stats()
        assert st["slots"] == 1 and st["max_slots_busy"] == 1
    # a budget of four slots: more slots join while requests wait
    with bwt.Server(hbm_budget=per * 4, max_slots=4, slot_bytes=slot_bytes, slot_blocks=16) as srv:
        _load(srv, blocks)
        assert srv.stats()["slots"] >= 2
    # a large budget, but the free HBM read at admission time covers no other
    # slot: the requests wait for the one slot; once memory is freed again the
    # server grows
    with bwt.Server(hbm_budget=per * 4, max_slots=4, slot_bytes=slot_bytes, slot_blocks=16) as srv:
        free, _ = torch.cuda.mem_get_info()
        hog = torch.empty(free - (256 << 20) - per // 2, dtype=torch.uint8, device="cuda")
        try:
            _load(srv, blocks)
            st = srv.stats()
            assert st["slots"] == 1 and st["admission_refused"] >= 1
        finally:
            del hog
            torch.cuda.empty_cache()
        _load(srv, blocks)
        assert srv.stats()["slots"] >= 2
