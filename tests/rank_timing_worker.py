"""One rank of tests/test_bench_ranks.py::test_gpu_arm_rank_timing: bench.py's
timing helpers under a gloo process group, with a timed region of a
different length on each rank."""
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
    bench.rank_barrier(dist)
    t_local = 0.5 + 1.5 * rank  # rank 1 is the slowest
    t_max = bench.max_over_ranks(t_local, dist)
    bench.rank_barrier(dist)
    mine = {"rank": rank, "world": world, "t_local": t_local, "t_max": t_max,
            "value": bench.job_throughput(world, 1000, 10, t_max)}
    every = [None] * world
    dist.all_gather_object(every, mine)
    if rank == 0:
        print(json.dumps(every), flush=True)
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
