"""Replica-parallel host logic under a real 2-rank gloo process group (CPU)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from lgt_gb300 import dist as D
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items = list(range(64))
    mine = D.shard(items, rank, world)
    t = 1.0 + rank          # pretend rank r took 1 + r seconds
    m = D.max_over_ranks(t)
    D.barrier()
    out.put((rank, mine, m, D.world()))
    dist.destroy_process_group()


def test_shard_partitions():
    from lgt_gb300 import dist as D
    for n in (0, 1, 7, 64, 65):
        for w in (1, 2, 3, 8):
            parts = [D.shard(list(range(n)), r, w) for r in range(w)]
            assert sum(parts, []) == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_two_rank_gloo_max_and_shards():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == list(range(32)) and res[1][1] == list(range(32, 64))
    assert res[0][2] == res[1][2] == pytest.approx(2.0)
    assert res[1][3] == (1, 2, 1)
