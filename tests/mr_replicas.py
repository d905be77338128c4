"""Two-rank check of bench.py's replica helpers (run under torchrun by
tests/test_multirank.py): gloo process group, barrier, max over ranks."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def main():
    world, rank, local = bench.dist_setup()
    bench.barrier(world)
    mine = 10.0 * (rank + 1)
    top = bench.max_over_ranks(world, mine)
    # one write() per line: both ranks share the pipe, and a write under PIPE_BUF is atomic
    line = json.dumps({"rank": rank, "local": local, "world": world, "mine": mine, "max": top}) + "\n"
    os.write(1, line.encode())
    import torch.distributed as dist
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
