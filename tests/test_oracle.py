"""The CPU oracle, pinned before it is trusted: golden vectors (definition-level
BWT, the reference's BSC test strings), brute-force suffix order, exhaustive
small alphabets, a second independent suffix sorter (prefix doubling) at
megabyte sizes, and the inverse."""
import itertools
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bwt_vectors.json")


def _vectors():
    with open(GOLDEN) as f:
        return json.load(f)["vectors"]


@pytest.mark.parametrize("vec", _vectors(), ids=lambda v: v["name"])
def test_oracle_matches_golden(oracle, vec):
    t = bytes.fromhex(vec["input"])
    u, idx, aux = oracle.bwt_encode(t, aux_rate=vec["aux_rate"]) if t else (np.zeros(0, np.uint8), 0, [])
    assert bytes(u) == bytes.fromhex(vec["bwt"])
    assert idx == vec["index"]
    if t:
        # oracle aux[0] is the primary index, then suffixes r, 2r, ...
        assert list(aux[1:]) == vec["aux"]
        assert aux[0] == idx
    assert bytes(oracle.bwt_decode(bytes.fromhex(vec["bwt"]), vec["index"])) == t


def test_textbook_banana(oracle):
    # banana$ -> annb$aa; libsais drops the sentinel and reports its row.
    u, idx = oracle.bwt_encode(b"banana")
    assert bytes(u) == b"annbaa" and idx == 4


def test_python_definition_agrees(oracle):
    rng = np.random.default_rng(7)
    for _ in range(40):
        t = bytes(rng.integers(0, int(rng.integers(1, 6)), int(rng.integers(1, 200))).astype(np.uint8))
        u, idx = oracle.bwt_encode(t)
        assert (bytes(u), idx) == oracle.naive_bwt(t)


def test_exhaustive_binary_alphabet(oracle):
    for n in range(1, 11):
        for bits in itertools.product(b"AC", repeat=n):
            t = bytes(bits)
            u, idx = oracle.bwt_encode(t)
            assert (bytes(u), idx) == oracle.naive_bwt(t)
            assert bytes(oracle.bwt_decode(u, idx)) == t


def test_suffix_array_vs_bruteforce(oracle):
    rng = np.random.default_rng(11)
    for _ in range(60):
        n = int(rng.integers(1, 3000))
        t = rng.integers(0, int(rng.choice([1, 2, 4, 256])), n).astype(np.uint8)
        assert (oracle.suffix_array(t) == oracle.suffix_array(t, brute=True)).all()


def test_decode_rejects_bad_index(oracle):
    u, idx = oracle.bwt_encode(b"ACGTTGCA")
    for bad in (0, -3, 9):
        with pytest.raises(ValueError):
            oracle.bwt_decode(u, bad)


def test_batch_matches_single(oracle):
    rng = np.random.default_rng(3)
    blocks = [rng.integers(0, 4, int(rng.integers(0, 5000))).astype(np.uint8) for _ in range(9)]
    us, idx = oracle.bwt_encode_batch(blocks, threads=4)
    for b, u, i in zip(blocks, us, idx):
        if len(b):
            uu, ii = oracle.bwt_encode(b)
            assert (u == uu).all() and i == ii
    back = oracle.bwt_decode_batch(us, idx, threads=4)
    assert all((x == y).all() for x, y in zip(back, blocks))


def test_doubling_agrees_with_bruteforce(oracle):
    rng = np.random.default_rng(31)
    for n in (1, 2, 3, 17, 100, 1000):
        for alpha in (1, 2, 4, 256):
            t = rng.integers(0, alpha, n).astype(np.uint8)
            assert (oracle.suffix_array(t, method="doubling") == oracle.suffix_array(t, brute=True)).all()


@pytest.mark.parametrize("kind", ["dna", "quality", "header", "repeat", "period3", "single", "random"])
def test_sais_agrees_with_doubling_at_megabytes(oracle, kind):
    # two independent suffix sorters agree at sizes brute force cannot reach
    from qz_gb300 import synth

    n = 1_500_000
    if kind == "dna":
        t = synth.sample_reads(synth.uniform_genome(200_000, seed=41), n // 150, seed=42)
    elif kind == "quality":
        t = synth.quality_stream(n // 132, seed=43)
    elif kind == "header":
        t = synth.header_stream(n // 45, seed=44)
    elif kind == "repeat":
        t = synth.sample_reads(synth.repeat_genome(100_000, seed=45), n // 250, seed=46, read_len=250)
    elif kind == "period3":
        t = np.resize(np.frombuffer(b"ACG", np.uint8), n)
    elif kind == "single":
        t = np.full(n, ord("N"), np.uint8)
    else:
        t = np.random.default_rng(47).integers(0, 256, n).astype(np.uint8)
    sa = oracle.suffix_array(t)
    assert (sa == oracle.suffix_array(t, method="doubling")).all()
    u, idx = oracle.bwt_encode(t)
    assert (oracle.bwt_decode(u, idx) == t).all()



def test_tuned_build_keeps_the_base_instruction_set():
    # The timed CPU baseline loads the tuned oracle on the GPU hosts, whose
    # kernels expose no SVE to user space: the aarch64 build may tune for the
    # core but must not select an instruction set beyond the base one (an
    # -mcpu=neoverse-v2 build emitted SVE and stopped with SIGILL there).
    mk = open(os.path.join(os.path.dirname(__file__), "..", "oracle", "Makefile")).read()
    arm = mk.split("ifeq ($(ARCH),aarch64)", 1)[1].split("else", 1)[0]
    tune = [ln.split(":=", 1)[1].split() for ln in arm.splitlines() if ln.strip().startswith("TUNE")]
    assert tune and all(f.startswith("-mtune=") for f in tune[0]), tune
    assert "-mcpu" not in mk.split("TUNED_CFLAGS", 1)[1].split("\n", 1)[0]
    assert "native" not in mk.split("TUNED_CFLAGS", 1)[1].split("\n", 1)[0]
