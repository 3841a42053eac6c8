"""One rank of the two-rank CPU check of bench.py's multi-rank logic
(gloo): reads RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT from the
environment, reduces a rank-dependent time over the ranks and prints the
slowest time and the whole-job value as JSON.  Run by
tests/test_bench_dist_cpu.py."""
import json
import os
import sys

import torch.distributed as dist

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import bench  # noqa: E402

rank, ws = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", rank=rank, world_size=ws)
ms = bench.max_over_ranks(10.0 + 5.0 * rank)
print(json.dumps({"rank": rank, "ms": ms, "value": bench.whole_job_value(1_000_000, ws, ms)}))
dist.barrier()
dist.destroy_process_group()
