"""The multi-rank path of bench.py on CPU: two gloo ranks (127.0.0.1) set up
as the launcher would, then the barrier, the max over ranks (the timing rule:
the slowest rank's time) and the sum over ranks (whole-job throughput)."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local = bench.dist_setup(2)
assert world == 2 and rank == int(os.environ["RANK"])
bench.barrier(world)
mx = bench.max_over_ranks(10.0 + rank, world)
sm = bench.sum_over_ranks(1.5 * (rank + 1), world)
print("rank", rank, "max", mx, "sum", sm, flush=True)
import torch.distributed as td
td.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_like_the_launcher():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    for rank, (o, _) in enumerate(outs):
        words = o.split()
        assert words[:2] == ["rank", str(rank)]
        assert float(words[3]) == 11.0   # the slowest rank's value
        assert float(words[5]) == 4.5    # 1.5 + 3.0


PARTITION_CHILD = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, os.path.join(sys.argv[1], "cuda-thermal_gb300"))
import bench
import torch.distributed as td
rank, world, local = bench.dist_setup(2)
import workloads
specs = workloads.batch_instance_specs(bench.BATCH_N, seed=bench.BATCH_SEED)
costs = [nx * ny * sum(l.ncells for l in cs.layers) for cs, nx, ny in specs]
mine = bench.partition_instances(costs, world)[rank]
got = [None] * world
td.all_gather_object(got, mine)
load = bench.sum_over_ranks(float(sum(costs[i] for i in mine)), world)
mx = bench.max_over_ranks(float(sum(costs[i] for i in mine)), world)
print("rank", rank, "n", len(mine), "union", sorted(i for p in got for i in p) == list(range(len(costs))),
      "disjoint", len(set(got[0]) & set(got[1])) == 0, "total", load == float(sum(costs)),
      "imbalance", mx - load / world <= max(costs), flush=True)
td.destroy_process_group()
"""


def test_batch_partition_covers_every_instance_once():
    """bench.py's batched run on two gloo ranks: each rank's cost-balanced
    share of the 256 instances, gathered, covers every instance exactly once,
    and the busiest rank carries at most one instance more than its share."""
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", PARTITION_CHILD, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=180) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    for rank, (o, _) in enumerate(outs):
        w = o.split()
        assert w[:2] == ["rank", str(rank)]
        assert w[5] == "True" and w[7] == "True" and w[9] == "True" and w[11] == "True", o
