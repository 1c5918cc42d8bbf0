"""The sub-batch plan of a batched call (qz_gb300/csrc/plan.h, plain C++), run
on the CPU through a small g++ driver: every block lands in exactly one
sub-batch of consecutive blocks, sizes respect the limits, sub-batches only
the full-capacity lane can hold come first, and the rest are taken largest
first."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "qz_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "plan.h"

// stdin: limit lane_bytes nb n[0] ... n[nb-1]; stdout: one line per sub-batch
// in the order the lanes take them: seq b0 b1 off bytes
int main() {
    long long limit, lane;
    int nb;
    if (std::scanf("%lld %lld %d", &limit, &lane, &nb) != 3) return 2;
    std::vector<int> n(nb);
    for (int i = 0; i < nb; ++i)
        if (std::scanf("%d", &n[i]) != 1) return 2;
    std::vector<qz::SubBatch> big, small;
    qz::plan_sub_batches(nb, n.data(), limit, lane, &big, &small);
    for (const auto* v : {&big, &small})
        for (const auto& s : *v) std::printf("%d %d %d %lld %lld\n", s.seq, s.b0, s.b1, s.off, s.bytes);
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("plan")
    src = d / "plan_driver.cpp"
    src.write_text(DRIVER)
    exe = d / "plan_driver"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def plan(driver, sizes, limit, lane):
    inp = f"{limit} {lane} {len(sizes)} " + " ".join(str(int(s)) for s in sizes)
    r = subprocess.run([driver], input=inp, capture_output=True, text=True, check=True)
    return [tuple(int(x) for x in ln.split()) for ln in r.stdout.splitlines()]


def check(sizes, subs, limit, lane):
    offs = np.concatenate([[0], np.cumsum(sizes)])
    assert [s[0] for s in subs] == list(range(len(subs)))  # seq = the order printed
    covered = sorted((b0, b1) for _, b0, b1, _, _ in subs)
    # every block in exactly one sub-batch, sub-batches contiguous
    assert covered[0][0] == 0 and covered[-1][1] == len(sizes)
    assert all(a[1] == b[0] for a, b in zip(covered, covered[1:]))
    for _, b0, b1, off, nbytes in subs:
        assert b1 > b0 and off == offs[b0] and nbytes == offs[b1] - offs[b0]
        assert nbytes <= limit or b1 == b0 + 1  # a larger block goes alone
    nbig = sum(1 for s in subs if s[4] > lane)
    assert all(s[4] > lane for s in subs[:nbig])  # the full-capacity lane's work first
    small = [s[4] for s in subs[nbig:]]
    assert small == sorted(small, reverse=True)  # then largest first


@pytest.mark.parametrize("seed", range(6))
def test_uneven_sizes(driver, seed):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1024), np.log(26_214_400), 256)).astype(np.int64)
    for limit, lane in ((16 << 20, 64 << 20), (64 << 20, 64 << 20), (1 << 20, 64 << 20)):
        check(sizes, plan(driver, sizes, limit, lane), limit, lane)


def test_block_above_lane_size_goes_first(driver):
    sizes = [3000, 80_000_000, 4000, 2_000_000, 5]
    subs = plan(driver, sizes, 64 << 20, 64 << 20)
    check(sizes, subs, 64 << 20, 64 << 20)
    assert (subs[0][1], subs[0][2]) == (1, 2)  # the 80 MB block


def test_single_and_empty_blocks(driver):
    assert plan(driver, [], 1 << 20, 1 << 20) == []
    sizes = [0, 0, 7, 0]
    subs = plan(driver, sizes, 1 << 20, 1 << 20)
    check(sizes, subs, 1 << 20, 1 << 20)
    assert len(subs) == 1
