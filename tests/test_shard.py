"""The N-rank split of a batch: complete, disjoint and cost-balanced, checked
with two gloo ranks on CPU exchanging their shares."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from scft_gb300 import workloads as W
from scft_gb300.shard import instance_cost, partition, shard


def test_partition_complete_disjoint_balanced():
    insts = W.batch_mixed(1000, seed=4)
    costs = [instance_cost(d) for d in insts]
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(1000))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= min(loads) + max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    insts = W.batch_mixed(300, seed=8)
    mine = shard(insts, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        out.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_the_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = gathered
    assert not set(a) & set(b)
    assert sorted(a + b) == list(range(300))
