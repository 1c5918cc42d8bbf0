"""Generates tests/golden/bwt_vectors.json (run here, where the reference tree is
mounted; the GPU machine only reads the committed JSON).

Inputs:
  * the literal round-trip strings of the reference's BSC unit tests
    (crates/qz-lib/src/compression/bsc.rs:442-499), read from that file;
  * edge cases the reference's integration tests exercise at block level
    (crates/qz-lib/tests/integration_test.rs:1313-1335: single base, all-N,
    mixed lengths), plus 0/1/2-byte blocks;
  * small seeded blocks of each stream type (DNA, packed quality, headers).
Outputs (U, primary index, auxiliary indexes at rate 4) come from the
definition-level BWT in pure Python (sort every suffix with an implicit
smallest end marker), independent of the C oracle.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from qz_gb300 import synth  # noqa: E402

# The reference tree's root comes from the command line (first argument) or
# the QZ_REFERENCE environment variable; the BSC wrapper sits below it.
BSC_RS = os.path.join("crates", "qz-lib", "src", "compression", "bsc.rs")


def reference_root(argv) -> str:
    root = argv[1] if len(argv) > 1 else os.environ.get("QZ_REFERENCE", "")
    if not root or not os.path.exists(os.path.join(root, BSC_RS)):
        raise SystemExit("usage: make_golden.py <reference tree root>  (or set QZ_REFERENCE); "
                         f"{BSC_RS} must exist below it")
    return root


def naive(t: bytes, rate: int = 4):
    n = len(t)
    if n == 0:
        return b"", 0, []
    order = sorted(range(n), key=lambda i: t[i:])
    out = bytearray([t[n - 1]])
    primary = -1
    aux = {}
    for j, p in enumerate(order):
        if p == 0:
            primary = j + 1
        else:
            out.append(t[p - 1])
        if p % rate == 0 and p > 0:
            aux[p // rate] = j + 1
    return bytes(out), primary, [aux[k] for k in sorted(aux)]


def reference_test_strings(root: str) -> list[bytes]:
    src = open(os.path.join(root, BSC_RS)).read()
    tests = src[src.index("mod tests"):]
    out = []
    # byte-string literals, joined across Rust's "\<newline><indent>" continuation
    for m in re.finditer(r'b"((?:[^"\\]|\\.)*)"', tests, re.S):
        s = re.sub(r"\\\n\s*", "", m.group(1))
        out.append(s.encode())
    return out


def main():
    cases = []
    for i, s in enumerate(reference_test_strings(reference_root(sys.argv))):
        cases.append((f"bsc_rs_test_{i}", s))
    cases += [
        ("empty", b""),
        ("one_byte", b"A"),
        ("two_bytes_sorted", b"AC"),
        ("two_bytes_rev", b"CA"),
        ("banana", b"banana"),
        ("all_N", b"N" * 150),
        ("single_base_reads", b"A" * 40 + b"C" * 40 + b"G" * 40 + b"T" * 40),
        ("mixed_lengths", b"ACGT" * 3 + b"ACG" * 5 + b"NNNN" + b"TTTTTTTTGCA" * 4),
        ("period3", b"ACG" * 200),
        ("binary_zeros", bytes(100)),
        ("all_bytes", bytes(range(256)) * 2),
    ]
    rng = np.random.default_rng(20240601)
    g = synth.uniform_genome(20_000, seed=11)
    dna = synth.sample_reads(g, 8, seed=12)
    cases.append(("dna_reads", bytes(dna)))
    q = synth.quality_stream(10, seed=13)
    cases.append(("quality_packed", bytes(q)))
    h = synth.header_stream(20, seed=14)
    cases.append(("headers", bytes(h)))
    for k in range(6):
        n = int(rng.integers(2, 600))
        sigma = int(rng.choice([2, 3, 5, 40, 256]))
        cases.append((f"random_{k}_sigma{sigma}", bytes(rng.integers(0, sigma, n).astype(np.uint8))))
    vectors = []
    for name, t in cases:
        u, p, aux = naive(t)
        vectors.append({"name": name, "input": t.hex(), "bwt": u.hex(), "index": p, "aux_rate": 4, "aux": aux})
    with open(os.path.join(HERE, "bwt_vectors.json"), "w") as f:
        json.dump({"convention": "libsais: U[0]=T[n-1], sentinel row dropped, index = 1 + rank(suffix 0)",
                   "generator": "tests/golden/make_golden.py", "vectors": vectors}, f, indent=1)
    print(f"wrote {len(vectors)} vectors")


if __name__ == "__main__":
    main()
