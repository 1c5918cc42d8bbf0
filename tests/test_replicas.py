"""The multi-GPU form is replicas (blocks are independent, no exchange step):
one process per GPU under torch.distributed.run, each running the same
per-GPU workload, the job timed by its slowest rank.  These tests run that
host logic as two gloo ranks on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, nproc=2, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def _json_lines(out: str):
    return [json.loads(ln) for ln in out.splitlines() if ln.startswith("{")]


def test_job_rate_counts_every_replica():
    # two replicas of 1 MB per step, 4 steps in 0.5 s: 16 MB/s for the job
    assert bench.job_rate(2, 1_000_000, 4, 0.5) == pytest.approx(16.0)
    assert bench.max_over_ranks([3, 1.5]) == [3.0, 1.5]  # one process: unchanged


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    r = _torchrun([os.path.join("tests", "replica_worker.py"), str(tmp_path)])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = {}
    for k in range(2):
        with open(tmp_path / f"rank{k}.json") as f:
            d = json.load(f)
        lines[d["rank"]] = d
    assert sorted(lines) == [0, 1]
    for d in lines.values():
        assert d["world"] == 2
        assert d["max"] == [200.0, 50.0]  # the slowest rank's figure, element-wise
        # 2 replicas x 1 MB x 4 steps in 0.2 s
        assert d["rate"] == pytest.approx(40.0)


def test_reference_arm_prints_once_under_torchrun():
    # the CPU arm runs on rank 0 only; the other rank exits 0 without work
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--config", "chunk", "--reads", "4000",
                   "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_cpu_sample_keeps_the_kind_mix_and_rotates_through_every_block():
    # the chunk's 15 sequence / 13 quality / 5 header blocks, 16 host cores
    kinds = ["seq"] * 15 + ["qual"] * 13 + ["hdr"] * 5
    blocks = [bytes([i]) for i in range(len(kinds))]
    seen = set()
    for step in range(5):
        ids, sample, skinds = bench.cpu_sample(blocks, kinds, 16, step=step)
        assert len(ids) == len(set(ids)) == 16 and ids == sorted(ids)
        assert [blocks[i] for i in ids] == sample and [kinds[i] for i in ids] == skinds
        # within one block of the workload's proportions for each kind
        for k, c in (("seq", 15), ("qual", 13), ("hdr", 5)):
            assert abs(skinds.count(k) - 16 * c / 33) <= 1.5
        seen.update(ids)
    assert seen == set(range(33))
    # both arms print the same config object for the same workload
    a = bench.workload_config("w", blocks, 1)
    assert a == bench.workload_config("w", blocks, 1) and a["blocks"] == 33 and a["bytes"] == 33
