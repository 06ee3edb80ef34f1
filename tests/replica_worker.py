"""One rank of the two-rank replica test (run by torchrun with the gloo
backend on 127.0.0.1; see test_replicas.py). Writes what this rank saw to
<out_dir>/rank<r>.json."""
import json
import os
import sys

import torch.distributed as dist

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "cdet-renyi-entanglement-hpc_gb300"))

from cdet_gb300 import replicas  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402


def main():
    out_dir = sys.argv[1]
    world, rank, local_rank = replicas.rank_info()
    dist.init_process_group("gloo")
    first = uniform_configurations(replicas.batch_seed(rank, 0), 4, 3)
    batches = [None] * world
    dist.all_gather_object(batches, first.tolist())
    slowest = replicas.max_over_ranks(1.0 + 0.5 * rank, world)  # rank r "took" 1 + r/2 s
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"world": world, "rank": rank, "local_rank": local_rank, "batches": batches,
                   "slowest": slowest,
                   "throughput": replicas.job_throughput(65536, 5, world, slowest)}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
