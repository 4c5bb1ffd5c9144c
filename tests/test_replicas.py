"""N>1 path: job sharding and timing reductions across world_size-2 gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from qed3_gb300 import replicas


def test_shard_covers_every_item_once():
    for n in (0, 1, 7, 64, 256):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in replicas.shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(replicas.shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine = list(replicas.shard(10, rank, world))
    t = 1.0 + rank  # a per-rank step time
    mx = replicas.max_over_ranks(t)
    total = replicas.sum_over_ranks(len(mine))
    replicas.barrier()
    out.put((rank, mine, mx, total))
    dist.destroy_process_group()


def test_gloo_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=60) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] + res[1][1] == list(range(10))
    assert res[0][2] == res[1][2] == 2.0
    assert res[0][3] == res[1][3] == 10.0
