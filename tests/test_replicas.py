"""Replica (N > 1) host logic with two gloo ranks on CPU: round-robin
sharding covers every unit once, and the job throughput uses the summed
units and the slowest rank's time."""
import os
import socket

import torch.multiprocessing as tmp

from pyhermes_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = replicas.shard(list(range(10)), rank, world)
    seconds = 1.0 + rank  # rank 1 is the slower one
    total, slowest, rate = replicas.job_throughput(len(units), seconds)
    q.put((rank, units, total, slowest, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_aggregate():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, u0, t0, s0, v0), (r1, u1, t1, s1, v1) = out
    assert sorted(u0 + u1) == list(range(10)) and not set(u0) & set(u1)
    assert t0 == t1 == 10.0 and s0 == s1 == 2.0 and v0 == v1 == 5.0


def test_single_process_passthrough():
    assert replicas.job_throughput(7, 2.0) == (7.0, 2.0, 3.5)
