"""Autotuner for the batched block-sorting path.

The library exposes runtime knobs per storage (qzgpu_storage_set_param):
sub-batch sizes of the forward and inverse lanes, persistent CTAs per SM of
the look-back radix passes, CTAs per SM of the one-CTA group sort, the longest
group sorted by one warp (the medium / tile class boundary), the inverse's
ruler stride, the look-back tile size of the large-group radix sort and the
width of its first digit (which decides three or four passes for 25..27-bit
rank keys).  The tuner times a forward + inverse of the caller's blocks for
candidate settings (coordinate descent from the defaults, best of `reps`
timings each) and keeps the fastest.  Results are cached in a JSON file per
workload signature: GPU name, block-size class and alphabet class.
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

SPACE = {
    "fwd_sub_bytes": [16 << 20, 32 << 20, 64 << 20],
    "inv_sub_bytes": [16 << 20, 32 << 20, 64 << 20],
    "big_ctas_per_sm": [2, 3, 4],
    "tile_ctas_per_sm": [1, 2, 3],
    "medium_max": [64, 128, 256, 512],
    "ruler_stride_log2": [4, 5, 6],
    "big_tile": [2048, 4096, 8192],
    "radix_first_bits": [8, 11],
    "round_pipeline": [0, 1],
    "split_lookback": [0, 1],
}


def cache_path() -> str:
    return os.environ.get("QZGPU_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "qz_gb300", "tune.json"))


def signature(blocks, gpu_name: str = "") -> str:
    """Block-size class (log2 of the mean block size) and alphabet class
    (distinct symbols of a sample: <=8 'dna', <=96 'text', else 'binary')."""
    sizes = [len(b) for b in blocks if len(b)]
    mean = sum(sizes) / max(len(sizes), 1)
    sample = np.concatenate([np.asarray(b[:65536]) for b in blocks[:64] if len(b)]) if sizes else np.zeros(1, np.uint8)
    sigma = len(np.unique(sample))
    alpha = "dna" if sigma <= 8 else ("text" if sigma <= 96 else "binary")
    return f"{gpu_name}|size2^{int(math.log2(max(mean, 1)))}|{alpha}|blocks{min(len(blocks), 1024).bit_length()}"


def load_cache() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(c: dict) -> None:
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(c, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def apply(storage, params: dict) -> None:
    for k, v in params.items():
        if k in SPACE:
            storage.set_param(k, int(v))


def tune(storage, run, key: str | None = None, reps: int = 3, use_cache: bool = True, log=None,
         min_gain: float = 0.02) -> dict:
    """Coordinate descent over SPACE.  `run()` performs one forward + inverse of
    the workload on `storage` and returns its duration in ms; each candidate
    keeps the best of `reps` runs, and replaces the current setting only if it
    is faster by more than `min_gain` (a step of the multi-lane engine varies
    by a few percent from run to run).  Returns the best parameters (already
    applied to the storage) and records them under `key`."""
    cache = load_cache() if use_cache else {}
    if key and use_cache and key in cache:
        best = cache[key]["params"]
        apply(storage, best)
        return dict(best)
    current = {k: storage.get_param(k) for k in SPACE}

    def measure(params):
        apply(storage, params)
        return min(run() for _ in range(reps))

    best_ms = measure(current)
    t0 = time.time()
    trials = 1
    for k, values in SPACE.items():
        for v in values:
            if v == current[k]:
                continue
            cand = dict(current, **{k: v})
            ms = measure(cand)
            trials += 1
            if log:
                log(f"autotune {k}={v}: {ms:.2f} ms (best {best_ms:.2f})")
            if ms < best_ms * (1.0 - min_gain):
                best_ms, current = ms, cand
    apply(storage, current)
    if key:
        cache = load_cache()
        cache[key] = {"params": current, "ms": best_ms, "trials": trials, "seconds": round(time.time() - t0, 1)}
        try:
            save_cache(cache)
        except OSError:
            pass
    return current
