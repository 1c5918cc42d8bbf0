"""Autotuner logic on the host (no GPU): coordinate descent keeps the fastest
setting of each knob and the cache round-trips."""
import numpy as np

from qz_gb300 import autotune


class FakeStorage:
    def __init__(self):
        self.p = {"fwd_sub_bytes": 64 << 20, "inv_sub_bytes": 64 << 20, "big_ctas_per_sm": 3,
                  "tile_ctas_per_sm": 3, "medium_max": 512, "ruler_stride_log2": 5, "big_tile": 4096,
                  "radix_first_bits": 11, "round_pipeline": 0, "split_lookback": 0}

    def set_param(self, k, v):
        self.p[k] = v

    def get_param(self, k):
        return self.p[k]


def test_coordinate_descent_finds_best(tmp_path, monkeypatch):
    monkeypatch.setenv("QZGPU_TUNE_CACHE", str(tmp_path / "tune.json"))
    st = FakeStorage()
    target = {"fwd_sub_bytes": 32 << 20, "big_ctas_per_sm": 3, "medium_max": 128, "ruler_stride_log2": 6,
              "big_tile": 8192, "radix_first_bits": 8}

    def run():
        # cost falls as each knob approaches its target value
        return 10.0 + sum(abs(np.log2(st.p[k]) - np.log2(v)) for k, v in target.items())

    best = autotune.tune(st, run, key="k1", reps=1)
    for k, v in target.items():
        assert best[k] == v
    assert st.p == best
    # cached: a fresh storage gets the same settings without timing
    st2 = FakeStorage()
    again = autotune.tune(st2, lambda: 1 / 0, key="k1", reps=1)
    assert again == best and st2.p == best


def test_signature_classes():
    dna = [np.frombuffer(b"ACGTN" * 1000, np.uint8)]
    txt = [np.frombuffer(bytes(range(32, 100)) * 100, np.uint8)]
    binary = [np.arange(65536, dtype=np.uint32).astype(np.uint8)]
    assert "|dna|" in autotune.signature(dna, "G")
    assert "|text|" in autotune.signature(txt, "G")
    assert "|binary|" in autotune.signature(binary, "G")
