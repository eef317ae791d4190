"""Replicas across ranks (world size 2, gloo on the CPU): every unit is served by exactly one rank,
and the report combines the slowest rank's time with the total work."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    from tropidist_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = replicas.shard(range(11), rank, world)
    ms, work = replicas.aggregate(10.0 + rank, len(units))
    q.put((rank, units, ms, work))
    dist.barrier()
    dist.destroy_process_group()


def test_shards_and_aggregate_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    units = out[0][1] + out[1][1]
    assert sorted(units) == list(range(11))
    for _, _, ms, work in out:
        assert ms == 11.0 and work == 11.0


def test_shard_single_rank_is_everything():
    from tropidist_gb300 import replicas
    assert replicas.shard(range(5), 0, 1) == list(range(5))
    assert replicas.aggregate(3.0, 7) == (3.0, 7.0)
