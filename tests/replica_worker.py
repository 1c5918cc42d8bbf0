"""One rank of the replica timing test, launched by torch.distributed.run with
the gloo backend (no GPU): each rank reports made-up per-rank timings, reduces
them with bench.max_over_ranks and writes the result as JSON to
<out_dir>/rank<r>.json (one file per rank: printed lines of two ranks can
interleave)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import torch.distributed as dist  # noqa: E402

import bench  # noqa: E402


def main():
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    # rank r is slow on the first figure and fast on the second
    mine = [100.0 * (rank + 1), 50.0 - rank]
    out = bench.max_over_ranks(mine, dist)
    rate = bench.job_rate(world, 1_000_000, 4, out[0] / 1e3)
    with open(os.path.join(sys.argv[1], f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "mine": mine, "max": out, "rate": rate}, f)
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
