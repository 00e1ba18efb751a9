"""World-size-2 gloo run of the multi-rank bookkeeping (CPU only): disjoint shards, max/sum agreement."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_units, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from lagrangian_microbes_gb300.replicas import max_over_ranks, shard, sum_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = list(shard(n_units, world, rank))
    fake_ms = 10.0 + 5.0 * rank  # each rank's timed region
    out[rank] = (mine, max_over_ranks(fake_ms), sum_over_ranks(len(mine)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, 256, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    a, b = out[0], out[1]
    assert set(a[0]).isdisjoint(b[0]) and sorted(a[0] + b[0]) == list(range(256))
    assert a[1] == b[1] == 15.0
    assert a[2] == b[2] == 256
