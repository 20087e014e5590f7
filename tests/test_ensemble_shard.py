"""Multi-GPU host logic on CPU: ensemble members shard across ranks with no
data-path collective; scalar diagnostics are gathered (gloo, world size 2)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from nspipe_gb300.ensemble import shard


@pytest.mark.parametrize("n,world", [(64, 1), (64, 2), (64, 3), (5, 8), (7, 2)])
def test_shards_partition_the_members(n, world):
    seen = []
    for r in range(world):
        lo, hi = shard(n, world, r)
        assert 0 <= lo <= hi <= n
        seen += list(range(lo, hi))
    assert seen == list(range(n))
    sizes = [shard(n, world, r)[1] - shard(n, world, r)[0] for r in range(world)]
    assert max(sizes) - min(sizes) <= 1


def test_shard_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "nspipe-gpu_gb300"))
    from nspipe_gb300.ensemble import gather_scalars, shard as sh
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = sh(n, world, rank)
    # each rank "advances" its own members: a per-member scalar that depends only on the member id
    vals = [float(m * m) for m in range(lo, hi)]
    got = gather_scalars(vals)
    dist.destroy_process_group()
    q.put((rank, got))


def test_gloo_two_ranks_gather_member_scalars():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port, n, world = _free_port(), 9, 2
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        flat = [v for part in res[r] for v in part]
        assert flat == [float(m * m) for m in range(n)]
