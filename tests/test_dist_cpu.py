"""The multi-rank bookkeeping of the benchmark on CPU with gloo, world size 2:
disjoint shards, disjoint ensemble seeds, max-over-ranks timing and summed
units."""
import os
import socket

import pytest

from abie_gb300 import dist as D


def test_shards_cover_disjointly():
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = D.shard(n, r, world)
                seen.extend(range(lo, hi))
            assert seen == list(range(n))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = D.rank_info()
    secs = 1.0 + r          # rank 1 is the slow one
    units = 100 * (r + 1)
    t, u = D.reduce_timing(secs, units)
    seed0 = D.ensemble_seed0(10000, r, 4096)
    out.put((r, w, t, u, seed0))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 2.0 and r[3] == 300.0 for r in res)   # max time, summed units
    assert res[0][4] == 10000 and res[1][4] == 14096            # disjoint systems
