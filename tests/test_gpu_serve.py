"""Serving form: concurrent mixed forward / inverse requests batched onto
resident slots give, request by request, the same result as the request run
alone (bit-exact)."""
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
        assert srv.slots >= 1
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
