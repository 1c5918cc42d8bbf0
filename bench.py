"""Benchmark of the GB300 block-sorting stage (forward + inverse BWT).

One step = forward BWT of every block of the workload followed by the inverse
BWT of the result, device-resident inputs (the round trip is checked on the
device after warm-up).  Default workload: one qz chunk of 2.5M synthetic
150 bp reads split into qz's sequence / quality / header streams and cut into
25 MiB blocks (33 blocks, 818 MB), all blocks in one batched call.

Beside the timed step the default line carries:
  * parity: the GPU's output of the blocks the CPU baseline sorted, compared
    with the oracle's (the run fails on a mismatch);
  * roofline of the dominant kernel (event-timed inside the timed region, and
    alone on a one-lane storage) and a clean per-kernel table from that
    one-lane pass;
  * e2e through the host-buffer C ABI (copies inside the timed region);
  * batched_vs_plain: the 256-block uneven batch (1 KB-25 MiB), autotuned
    batched calls against one call per block on the same inputs;
  * serving: saturation MB/s and p50/p99 latency at 0.5x / 1.0x / 1.5x load.

Prints one JSON line (rank 0).  `--impl reference` times the CPU path instead
(the C oracle built with -O3 and host-core tuning, one block per host thread as
qz runs libbsc under rayon), each step on a bounded, kind-stratified sample of
the same workload that rotates through all its blocks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "BSC BWT fwd/inv MB/s on 1 GB300, batched+served p50/p99 vs plain kernel & CPU"
FALLBACK_HBM_GBS = 6800.0


# --------------------------------------------------------------------------- workload


def make_workload(name: str, reads: int):
    from qz_gb300 import synth

    if name == "chunk":
        blocks = synth.chunk_blocks(reads)
        desc = f"one qz chunk: {reads} x 150 bp synthetic reads -> seq/qual/header streams, 25 MiB blocks"
    elif name == "plain":
        blocks = [("seq", synth.plain_block())]
        desc = "one 24,999,900-byte sequence block (166,666 x 150 bp reads, 5 Mbp genome)"
    elif name == "uneven":
        blocks = synth.uneven_blocks(256)
        desc = "256 blocks, sizes log-uniform 1 KB-25 MiB, 50% DNA / 30% quality / 20% header"
    elif name == "ultra":
        blocks = [("seq", synth.ultra_block())]
        desc = "one 750 MiB ultra-mode sequence block (150 bp reads, 50 Mbp genome)"
    elif name == "repeat":
        blocks = synth.repeat_blocks()
        desc = "repeat-rich: 250 bp reads at 30x over 1 Mbp with 20% tandem repeats, one single-byte and one period-3 block"
    else:
        raise SystemExit(f"unknown config {name}")
    return [b for _, b in blocks], [k for k, _ in blocks], desc


def workload_config(desc: str, blocks, world: int) -> dict:
    """The `config` object both arms print for the same workload."""
    return {"workload": desc, "blocks": len(blocks), "bytes": int(sum(len(b) for b in blocks)),
            "l2": "inputs larger than L2 (workload bytes and scratch exceed 126 MB)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "step": "forward BWT of all blocks + inverse BWT of the result"}


# --------------------------------------------------------------------------- clocks


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


# --------------------------------------------------------------------------- CPU path


def stratified_order(kinds) -> list[int]:
    """Block order that interleaves the kinds in the workload's proportions
    (block i of a kind with c blocks sits at (i + 0.5) / c), so that any run of
    consecutive entries has about the workload's kind mix."""
    seen, pos = {}, []
    count = {k: kinds.count(k) for k in set(kinds)}
    for i, k in enumerate(kinds):
        j = seen.get(k, 0)
        seen[k] = j + 1
        pos.append(((j + 0.5) / count[k], i))
    return [i for _, i in sorted(pos)]


def cpu_sample(blocks, kinds, cores: int, step: int = 0):
    """Step `step`'s bounded sample: `cores` blocks (one per host thread),
    consecutive in the stratified order and rotating with the step, so that
    successive steps cover every block of the workload."""
    order = stratified_order(kinds)
    take = max(1, min(len(blocks), cores))
    idx = sorted(order[(step * take + j) % len(order)] for j in range(take))
    return idx, [blocks[i] for i in idx], [kinds[i] for i in idx]


def time_cpu(sample, cores: int):
    """Oracle forward + inverse of the sample over `cores` host threads (the
    host-tuned build).  Returns (forward s, inverse s, U list, indexes)."""
    from oracle import oracle as O

    O.build()
    t0 = time.perf_counter()
    us, idx = O.bwt_encode_batch(sample, threads=cores, tuned=True)
    t1 = time.perf_counter()
    back = O.bwt_decode_batch(us, idx, threads=cores, tuned=True)
    t2 = time.perf_counter()
    for a, b in zip(back, sample):
        if not np.array_equal(a, b):
            raise SystemExit("CPU round trip mismatch")
    return t1 - t0, t2 - t1, us, [int(i) for i in idx]


def cpu_desc(sample, kinds) -> str:
    mb = sum(len(b) for b in sample) / 1e6
    mix = {k: kinds.count(k) for k in sorted(set(kinds))}
    return f"{len(sample)} blocks ({mb:.1f} MB; " + ", ".join(f"{v} {k}" for k, v in mix.items()) + ")"


CPU_BUILD = "C oracle (SA-IS + LF inverse), gcc -O3 tuned for the host core; oracle CPU, not libbsc"


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    blocks, kinds, desc = make_workload(args.config, args.reads)
    cores = os.cpu_count() or 1
    for w in range(args.warmup):
        _, sample, _ = cpu_sample(blocks, kinds, cores, step=w)
        time_cpu(sample, cores)
    times, nbytes, covered = [], 0, set()
    mix = []
    for k in range(args.steps):
        ids, sample, skinds = cpu_sample(blocks, kinds, cores, step=args.warmup + k)
        te, ti, _, _ = time_cpu(sample, cores)
        times.append(te + ti)
        nbytes += sum(len(b) for b in sample)
        covered.update(ids)
        mix += skinds
    total = sum(times)
    value = nbytes / total / 1e6
    per_step = nbytes / args.steps
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "MB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": workload_config(desc, blocks, world),
        "cpu_baseline": {"value": round(value, 3), "unit": "MB/s", "cores": cores, "kind": "port",
                         "sample": (f"each step {min(cores, len(blocks))} of the {len(blocks)} blocks "
                                    f"({per_step / 1e6:.1f} MB), one per host thread, consecutive in a "
                                    f"kind-stratified order that rotates with the step; {len(covered)} of "
                                    f"{len(blocks)} blocks covered, timed mix "
                                    + ", ".join(f"{mix.count(k)} {k}" for k in sorted(set(mix)))
                                    + f"; forward + inverse; {CPU_BUILD} (libbsc is not in the reference tree)"),
                         "cpu": cpu_model()},
        "e2e": {"value": round(value, 3), "unit": "MB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- replicas


def max_over_ranks(values, dist=None):
    """Per-rank timings reduced element-wise to the slowest rank's (gloo
    all-reduce MAX): the job takes as long as its slowest replica."""
    vals = [float(v) for v in values]
    if dist is None:
        return vals
    import torch

    t = torch.tensor(vals, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_rate(world: int, nbytes: int, steps: int, seconds: float) -> float:
    """Whole-job MB/s: each of `world` replicas processes the same `nbytes`
    per step (weak scaling), timed by the slowest rank."""
    return world * nbytes * steps / seconds / 1e6


# --------------------------------------------------------------------------- GPU path


def load_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def load_traffic():
    """Per-launch DRAM bytes of kernels from a committed ncu summary, if any:
    {kernel: {"dram_bytes_per_launch", "alg_bytes_per_launch", ...}}."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def one_lane_storage(bwt, nbytes, nblocks, tuned, params):
    old = os.environ.get("QZGPU_LANES")
    os.environ["QZGPU_LANES"] = "1"
    try:
        st1 = bwt.Storage(nbytes, nblocks)
    finally:
        if old is None:
            del os.environ["QZGPU_LANES"]
        else:
            os.environ["QZGPU_LANES"] = old
    for k, v in (tuned or {}).items():
        if k in bwt.Storage.PARAMS:  # settable knobs only ("lanes" is read-only)
            st1.set_param(k, int(v))
    for kv in params:
        k, v = kv.split("=", 1)
        st1.set_param(k, int(v))
    return st1


def autotune_storage(st, step, blocks, dev, stream, reps=3):
    import torch

    from qz_gb300 import autotune

    def run_once():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1)

    run_once()
    key = autotune.signature(blocks, torch.cuda.get_device_name(dev))
    return autotune.tune(st, run_once, key=key, use_cache=False, reps=reps)


def batched_vs_plain(args, dev, stream):
    """The uneven batch (256 blocks, 1 KB-25 MiB, DNA / quality / header):
    autotuned batched calls against one forward + inverse call per block, on
    the same device-resident inputs."""
    import torch

    from qz_gb300 import bwt

    blocks, _, desc = make_workload("uneven", args.reads)
    sizes = [len(b) for b in blocks]
    N = sum(sizes)
    d_T = torch.from_numpy(np.concatenate(blocks)).to(dev)
    d_U = torch.empty_like(d_T)
    d_R = torch.empty_like(d_T)
    sptr = stream.cuda_stream
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    with bwt.Storage(N, len(blocks)) as st:
        def step():
            idx = st.encode_device(sizes, d_T.data_ptr(), d_U.data_ptr(), sptr)
            st.decode_device(sizes, idx, d_U.data_ptr(), d_R.data_ptr(), sptr)

        def plain_step():
            for b, n in enumerate(sizes):
                o = int(offs[b])
                ix = st.encode_device([n], d_T.data_ptr() + o, d_U.data_ptr() + o, sptr)
                st.decode_device([n], ix, d_U.data_ptr() + o, d_R.data_ptr() + o, sptr)

        tuned = None if args.no_autotune else autotune_storage(st, step, blocks, dev, stream, reps=2)

        def timed(fn, steps):
            for _ in range(3):
                fn()
            torch.cuda.synchronize(dev)
            d_R.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if not torch.equal(d_R, d_T):
                raise SystemExit("uneven batch round trip mismatch")
            return e0.elapsed_time(e1) / steps

        bms = timed(step, max(args.steps // 2, 3))
        pms = timed(plain_step, 2)
    return {"workload": desc, "blocks": len(blocks), "bytes": N,
            "batched_mb_s": round(N / bms / 1e3, 3), "batched_ms_per_step": round(bms, 3),
            "plain_mb_s": round(N / pms / 1e3, 3), "plain_ms_per_step": round(pms, 3),
            "batched_over_plain": round(pms / bms, 3), "tuned": tuned,
            "plain_path": "one qzgpu_bwt_encode_device + qzgpu_bwt_decode_device call per block",
            "step": "forward + inverse of every block, device-resident"}


def serve_sweep(nreq: int, loads, warmup: int, slots: int):
    """Poisson arrivals of block requests (70% forward, 30% inverse of blocks
    produced beforehand), sizes log-uniform 64 KiB-25 MiB, mixed DNA / quality /
    header content, served by qzgpu_server_* with continuous batching.  Returns
    the saturation point (all requests at once) and one point per offered
    load (a fraction of the saturation rate)."""
    from qz_gb300 import bwt, synth

    reqs = synth.serving_requests(nreq, rate_per_s=1.0, seed=6)
    inv_in = {}
    inv_ids = [i for i, r in enumerate(reqs) if r[1] == "inv"]
    with bwt.Storage(256 << 20, 256) as st:  # the inverse requests' inputs, made before timing
        chunk, used = [], 0
        for i in inv_ids + [None]:
            if i is None or used + len(reqs[i][3]) > (256 << 20):
                if chunk:
                    us, ix = st.encode_batch([reqs[j][3] for j in chunk])
                    for j, u, p in zip(chunk, us, ix):
                        inv_in[j] = (u, p)
                chunk, used = [], 0
            if i is not None:
                chunk.append(i)
                used += len(reqs[i][3])
    total_bytes = sum(len(r[3]) for r in reqs)
    mean_bytes = total_bytes / len(reqs)
    srv = bwt.Server(hbm_budget=0, max_slots=slots, slot_bytes=64 << 20, slot_blocks=256)

    def submit(i):
        _, op, _, block = reqs[i]
        if op == "inv":
            u, p = inv_in[i]
            return srv.submit_inverse(u, p)
        return srv.submit_forward(block)

    def run_point(gaps):
        tickets = [None] * len(reqs)
        lat = []
        done = threading.Event()

        def waiter():
            for i in range(len(reqs)):
                while tickets[i] is None:
                    time.sleep(0.0002)
                r = srv.wait(tickets[i])
                lat.append(r["latency_ms"])
            done.set()

        th = threading.Thread(target=waiter, daemon=True)
        th.start()
        t0 = time.perf_counter()
        nxt = t0
        for i in range(len(reqs)):
            if gaps is not None:
                nxt += gaps[i]
                d = nxt - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            tickets[i] = submit(i)
        done.wait()
        t1 = time.perf_counter()
        lat.sort()
        return {"mb_s": round(total_bytes / (t1 - t0) / 1e6, 3),
                "p50_ms": round(lat[len(lat) // 2], 3), "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
                "wall_s": round(t1 - t0, 3)}

    try:
        for _ in range(max(1, warmup)):
            run_point(None)
        sat = run_point(None)
        sat_rate = sat["mb_s"] * 1e6 / mean_bytes  # requests per second at saturation
        rng = np.random.default_rng(60)
        unit_gaps = rng.exponential(1.0, len(reqs))
        points = []
        for frac in loads:
            pt = run_point(unit_gaps / (frac * sat_rate))
            pt["offered_load"] = frac
            pt["offered_mb_s"] = round(frac * sat["mb_s"], 3)
            points.append(pt)
        stats = srv.stats()
    finally:
        srv.close()
    return {"requests": len(reqs), "bytes_per_point": total_bytes, "saturation": sat, "load_points": points,
            "server": stats}


def run_gpu(args, rank: int, world: int):
    import torch

    from qz_gb300 import bwt

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    blocks, kinds, desc = make_workload(args.config, args.reads)
    sizes = [len(b) for b in blocks]
    N = sum(sizes)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    host = np.concatenate(blocks)
    dev = torch.device("cuda", local)
    d_T = torch.from_numpy(host).to(dev)
    d_U = torch.empty_like(d_T)
    d_R = torch.empty_like(d_T)
    bwt.init()
    st = bwt.Storage(N, len(blocks))
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step():
        idx = st.encode_device(sizes, d_T.data_ptr(), d_U.data_ptr(), sptr)
        st.decode_device(sizes, idx, d_U.data_ptr(), d_R.data_ptr(), sptr)
        return idx

    for kv in args.param:
        k, v = kv.split("=", 1)
        st.set_param(k, int(v))
    # ---- autotuner (before warm-up; not timed)
    tuned = None
    if not args.no_autotune:
        tuned = autotune_storage(st, step, blocks, dev, stream)
    for _ in range(args.warmup):
        idx = step()
    torch.cuda.synchronize(dev)
    if not torch.equal(d_R, d_T):
        raise SystemExit("GPU round trip mismatch")

    # ---- per-kernel table and the dominant kernel: one forward + inverse on a
    # one-lane storage, every launch bracketed by events (nothing else runs on
    # the GPU meanwhile, so each window is that kernel's own duration); not
    # part of the timed region
    peak, peak_kind = load_peak()
    st1 = one_lane_storage(bwt, N, len(blocks), tuned or st.params(), args.param)
    i1 = st1.encode_device(sizes, d_T.data_ptr(), d_U.data_ptr(), sptr)
    st1.decode_device(sizes, i1, d_U.data_ptr(), d_R.data_ptr(), sptr)
    st1.profile(True)
    st1.profile_read(reset=True)
    i1 = st1.encode_device(sizes, d_T.data_ptr(), d_U.data_ptr(), sptr)
    st1.decode_device(sizes, i1, d_U.data_ptr(), d_R.data_ptr(), sptr)
    torch.cuda.synchronize(dev)
    prof_all = st1.profile_read(reset=True)
    st1.profile(False)
    st1.close()
    dominant = prof_all[0]["name"] if prof_all else None
    kern_total = max(sum(q["ms"] for q in prof_all), 1e-9)
    kernels = []
    for p in prof_all:
        gbs = (p["alg_bytes"] / (p["ms"] / 1e3) / 1e9) if p["ms"] > 0 and p["alg_bytes"] > 0 else None
        kernels.append({"name": p["name"], "launches": p["launches"], "ms": round(p["ms"], 3),
                        "share": round(p["ms"] / kern_total, 4), "alg_gb_s": round(gbs, 1) if gbs else None})

    # ---- timed region (device-resident inputs, 818 MB > 126 MB L2); only the
    # dominant kernel's launches carry events, for the roofline
    clocks = ClockSampler(local)
    st.profile(True, only=dominant)
    st.profile_read(reset=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    time.sleep(0.3)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps + 1)]
    launches = 0
    fwd_stats, rounds_active = None, None
    ev[0].record(stream)
    for k in range(args.steps):
        idx = st.encode_device(sizes, d_T.data_ptr(), d_U.data_ptr(), sptr)
        fwd_stats = st.stats()
        rounds_active = st.round_counts()
        launches += fwd_stats["kernel_launches"]
        ev[2 * k + 1].record(stream)
        st.decode_device(sizes, idx, d_U.data_ptr(), d_R.data_ptr(), sptr)
        launches += st.stats()["kernel_launches"]
        ev[2 * k + 2].record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    if dist:
        dist.barrier()
    total_ms = ev[0].elapsed_time(ev[2 * args.steps])
    fwd_ms = sum(ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps))
    inv_ms = sum(ev[2 * k + 1].elapsed_time(ev[2 * k + 2]) for k in range(args.steps))
    prof_top = st.profile_read(reset=True)
    st.profile(False)
    total_ms, fwd_ms, inv_ms = max_over_ranks([total_ms, fwd_ms, inv_ms], dist)
    value = job_rate(world, N, args.steps, total_ms / 1e3)
    if not torch.equal(d_R, d_T):
        raise SystemExit("GPU round trip mismatch in the timed region")

    # ---- roofline of the dominant kernel
    top = prof_top[0] if prof_top else None
    roof = None
    if top:
        per_launch = top["alg_bytes"] / max(top["launches"], 1)
        avg_s = top["ms"] / max(top["launches"], 1) / 1e3
        achieved = per_launch / avg_s / 1e9 if avg_s > 0 else 0.0
        roof = {"bound": "hbm", "kernel": top["name"], "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "alg_bytes_per_launch": int(per_launch), "launches_timed": top["launches"],
                "how": "algorithmic bytes per launch / event-timed launch duration inside the timed region "
                       "(the engine's lanes overlap, so a window also holds other lanes' kernels)",
                "traffic": None}
        tr = load_traffic().get(top["name"])
        if isinstance(tr, dict) and tr.get("alg_bytes_per_launch"):
            # DRAM bytes measured by ncu on a smaller case at the same
            # sub-batch size, scaled to this launch by its algorithmic bytes
            ratio = tr["dram_bytes_per_launch"] / tr["alg_bytes_per_launch"]
            roof["traffic"] = int(ratio * per_launch)
            roof["traffic_over_alg"] = round(ratio, 3)
            roof["traffic_source"] = tr.get("source", "profiles/dram_traffic.json")
        alone = next((p for p in prof_all if p["name"] == top["name"]), None)
        if alone and alone["launches"] and alone["ms"] > 0:
            a1 = alone["alg_bytes"] / alone["launches"] / (alone["ms"] / alone["launches"] / 1e3) / 1e9
            roof["alone"] = {"achieved": round(a1, 1), "frac": round(a1 / peak, 4), "launches": alone["launches"],
                             "how": "one forward + inverse of the workload on a one-lane storage"}

    # ---- end to end through the host-buffer C ABI (copies inside the timed region)
    e2e = None
    if not args.no_e2e:
        # pinned host buffers, allocated once and reused by every step: the
        # step's inputs are copied to the device and its outputs back inside
        # the library calls
        def pinned(n):
            return torch.empty(max(n, 1), dtype=torch.uint8, pin_memory=True).numpy()[:n]

        h_in = [pinned(len(b)) for b in blocks]
        for h, b in zip(h_in, blocks):
            h[:] = b
        h_u = [pinned(len(b)) for b in blocks]
        h_back = [pinned(len(b)) for b in blocks]
        for _ in range(2):
            us, ix = st.encode_batch(h_in, out=h_u)
            st.decode_batch(h_u, ix, out=h_back)
        if dist:
            dist.barrier()
        fwd_s = inv_s = 0.0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ta = time.perf_counter()
            us, ix = st.encode_batch(h_in, out=h_u)
            tb = time.perf_counter()
            back = st.decode_batch(h_u, ix, out=h_back)
            fwd_s += tb - ta
            inv_s += time.perf_counter() - tb
        t1 = time.perf_counter()
        if not all(np.array_equal(a, b) for a, b in zip(back, blocks)):
            raise SystemExit("host round trip mismatch")
        e2e_s, fwd_s, inv_s = max_over_ranks([t1 - t0, fwd_s, inv_s], dist)
        e2e = {"value": round(job_rate(world, N, args.steps, e2e_s), 3), "unit": "MB/s",
               "h2d_bytes_per_step": 2 * N, "d2h_bytes_per_step": 2 * N,
               "fwd_ms_per_step": round(fwd_s / args.steps * 1e3, 3),
               "inv_ms_per_step": round(inv_s / args.steps * 1e3, 3),
               "api": "qzgpu_bwt_encode_batch + qzgpu_bwt_decode_batch (pinned host buffers, reused)"}
    st.close()

    # ---- CPU baseline on a bounded sample (rank 0, N=1 only), and parity of
    # the GPU's output of the same blocks against it
    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        ids, sample, skinds = cpu_sample(blocks, kinds, cores)
        te, ti, ous, oidx = time_cpu(sample, cores)
        cpu = {"value": round(sum(len(b) for b in sample) / (te + ti) / 1e6, 3), "unit": "MB/s", "cores": cores,
               "kind": "port", "sample": cpu_desc(sample, skinds) + f", one per host thread; forward + inverse; "
                                                                     f"{CPU_BUILD}",
               "fwd_mb_s": round(sum(len(b) for b in sample) / te / 1e6, 3),
               "inv_mb_s": round(sum(len(b) for b in sample) / ti / 1e6, 3), "cpu": cpu_model()}
        gu = d_U.cpu().numpy()
        bad = [i for j, i in enumerate(ids)
               if idx[i] != oidx[j] or not np.array_equal(gu[offs[i]:offs[i + 1]], ous[j])]
        parity = {"blocks": len(ids), "bytes": int(sum(len(b) for b in sample)), "bit_exact": not bad,
                  "against": "C oracle (SA-IS), U bytes and primary index of each block from the timed region's "
                             "last forward call"}
        if bad:
            print(json.dumps({"parity": parity, "mismatched_blocks": bad}), file=sys.stderr, flush=True)
            raise SystemExit(f"GPU output differs from the oracle in blocks {bad}")

    # ---- batched vs plain on the uneven batch, and the serving sweep (rank 0,
    # one GPU: sub-records beside the headline, not part of its timing)
    bvp, serving = None, None
    if rank == 0 and world == 1 and args.config == "chunk":
        del d_T, d_U, d_R
        torch.cuda.empty_cache()
        if not args.no_plain_compare:
            bvp = batched_vs_plain(args, dev, stream)
        if not args.no_serve:
            sv = serve_sweep(120, (0.5, 1.0, 1.5), warmup=1, slots=args.slots)
            serving = {"workload": "120 requests, Poisson arrivals, 70% forward / 30% inverse, sizes log-uniform "
                                   "64 KiB-25 MiB, 50% DNA / 30% quality / 20% header",
                       "saturation_mb_s": sv["saturation"]["mb_s"],
                       "points": [{k: p[k] for k in ("offered_load", "mb_s", "p50_ms", "p99_ms")}
                                  for p in sv["load_points"]],
                       "slots": sv["server"]["slots"], "batches": sv["server"]["batches"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "MB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded reads of the workload's shape; no public dataset)",
            "config": workload_config(desc, blocks, world),
            "tuned": tuned if tuned else None,
            "fwd_mb_s": round(job_rate(world, N, args.steps, fwd_ms / 1e3), 3),
            "inv_mb_s": round(job_rate(world, N, args.steps, inv_ms / 1e3), 3),
            "rounds": fwd_stats["rounds"] if fwd_stats else None,
            "active_per_round": rounds_active,
            "gpu_launches": launches,
            "parity": parity,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "kernels": kernels[:14], "kernels_note": "one forward + inverse on a one-lane storage, events around "
                                                     "every launch (not the timed region)",
            "batched_vs_plain": bvp, "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# --------------------------------------------------------------------------- serving


def run_serve(args, rank: int, world: int):
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from qz_gb300 import bwt

    bwt.init()
    sv = serve_sweep(args.requests, (0.25, 0.5, 0.75, 1.0, 1.25, 1.5), warmup=args.warmup, slots=args.slots)
    sat = sv["saturation"]
    if rank == 0:
        at1 = [p for p in sv["load_points"] if p["offered_load"] == 1.0][0]
        line = {
            "metric": METRIC, "value": sat["mb_s"], "unit": "MB/s", "n_gpus": world, "steps": len(sv["load_points"]),
            "warmup": max(1, args.warmup), "ms_per_step": round(1e3 * sat["wall_s"], 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded reads of the workload's shape; no public dataset)",
            "config": {"workload": f"serving: {sv['requests']} requests, Poisson arrivals, 70% forward / 30% inverse, "
                                   "sizes log-uniform 64 KiB-25 MiB, 50% DNA / 30% quality / 20% header",
                       "bytes_per_point": sv["bytes_per_point"], "slots": sv["server"]["slots"]},
            "saturation": sat, "p50_ms_at_saturation_load": at1["p50_ms"], "p99_ms_at_saturation_load": at1["p99_ms"],
            "load_points": sv["load_points"], "server": sv["server"],
        }
        print(json.dumps(line), flush=True)


def run_streams(args, rank: int):
    """Stream building on the device: one qz chunk's FASTQ text (2.5M x 150 bp
    reads) -> header / sequence / quality streams through qzgpu_fastq_streams
    (host buffers in and out, pinned and reused; copies inside the timed
    region).  CPU side: the Python oracle on a bounded sample of records."""
    import torch

    from qz_gb300 import bwt
    from qz_gb300 import streams as G
    from qz_gb300 import synth

    if rank != 0:
        return
    text = synth.chunk_fastq(args.reads)
    n = len(text)
    bwt.init()
    pin = torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy()
    pin[:] = text
    h, s, q, info = G.fastq_streams(pin)
    out = tuple(torch.empty(max(len(x), 1), dtype=torch.uint8, pin_memory=True).numpy()[: len(x)] for x in (h, s, q))
    for _ in range(args.warmup):
        G.fastq_streams(pin, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        G.fastq_streams(pin, out=out)
    dt = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import streams as S

        k = min(len(text), 200_000 * 360)
        sample = bytes(text[:k])
        cut = sample.rfind(b"\n@SIM") + 1  # whole records only
        t1 = time.perf_counter()
        S.fastq_streams(sample[:cut])
        c = time.perf_counter() - t1
        cpu = {"value": round(cut / c / 1e6, 3), "unit": "MB/s", "cores": 1, "kind": "port",
               "sample": f"first {cut} bytes of the text; Python oracle, not qz's Rust"}
    line = {"metric": "FASTQ -> qz streams MB/s (FASTQ bytes) on 1 GB300", "value": round(n / dt / 1e6, 3),
            "unit": "MB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8", "data": "synthetic (the chunk workload's reads as FASTQ text)",
            "config": {"workload": f"one qz chunk as FASTQ: {args.reads} x 150 bp reads, {n} bytes",
                       "path": "qzgpu_fastq_streams, pinned host buffers reused"},
            "streams": {k: v for k, v in info.items()}, "e2e": {"value": round(n / dt / 1e6, 3), "unit": "MB/s",
                                                               "h2d_bytes_per_step": n,
                                                               "d2h_bytes_per_step": len(h) + len(s) + len(q)},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="chunk", choices=["chunk", "plain", "uneven", "repeat", "ultra", "serve", "streams"])
    ap.add_argument("--requests", type=int, default=300, help="serve: requests per load point")
    ap.add_argument("--slots", type=int, default=4, help="serve: most device slots (admitted by free HBM)")
    ap.add_argument("--reads", type=int, default=2_500_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default knobs")
    ap.add_argument("--no-plain-compare", action="store_true", help="skip the uneven batched-vs-plain sub-record")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving sub-record")
    ap.add_argument("--param", action="append", default=[], metavar="NAME=VALUE",
                    help="set a storage knob (qzgpu_storage_set_param) before timing; repeatable")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config == "serve":
        run_serve(args, rank, world)
    elif args.config == "streams":
        run_streams(args, rank)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
