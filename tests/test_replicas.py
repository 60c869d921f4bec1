"""Host logic of the multi-rank (replicas-only) path, on CPU with gloo, world 2."""
import os

import pytest
import torch.multiprocessing as mp

from newrecon_gb300 import replicas


def test_shard_covers_every_case_once():
    items = list(range(16))
    got = []
    for r in range(3):
        got += replicas.shard(items, r, 3)
    assert sorted(got) == items
    assert replicas.shard(items, 1, 4) == [1, 5, 9, 13]
    with pytest.raises(ValueError):
        replicas.shard(items, 2, 2)


def test_case_seeds_distinct():
    seeds = {replicas.case_seed(0, r, c) for r in range(8) for c in range(16)}
    assert len(seeds) == 128


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, _ = replicas.env()
        mine = replicas.shard(list(range(10)), r, ws)
        # rank 1 is the slower one; units are the cases each rank processed
        el, units = replicas.reduce_timing(1.0 + r, float(len(mine)))
        q.put((r, el, units, mine))
    finally:
        dist.destroy_process_group()


def test_reduce_timing_gloo_world2():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for r, el, units, mine in res:
        assert el == 2.0          # max over ranks
        assert units == 10.0      # every case counted once
    assert sorted(res[0][3] + res[1][3]) == list(range(10))


def test_reduce_timing_single_process_is_identity():
    assert replicas.reduce_timing(1.5, 7) == (1.5, 7.0)
