"""Worker for tests/test_replicas_cpu.py, launched by torch.distributed.run
with the gloo backend on CPU: each rank reports a different step time, and
the bench's reduction must hand every rank the slowest one; rank 0 prints
the whole-job value as one JSON line."""
import json
import os
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import torch.distributed as dist  # noqa: E402

import bench  # noqa: E402


def main():
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    t = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    dist.barrier()
    if rank == 0:
        print(json.dumps({"world": world, "t_ms": t,
                          "value": bench.whole_job_gkeys(1 << 20, world, t),
                          "env_world": int(os.environ["WORLD_SIZE"])}), flush=True)
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
