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


# ---- a sharded run equals the single-rank run: each gloo rank steps its own members
# with the CPU oracle (FP64, one thread) through ShardedEnsemble, the same driver code
# that steps GPU members through nspipe_gb300.Stepper.

SHARD_CFG = (24, 8, 9, 1000.0, 0.01, 6.283185307179586)  # NR, NT, NZ, Re, dt, LZ (small s1 pipes)
SHARD_N, SHARD_STEPS = 5, 3


class OracleStepper:
    """The stepper protocol of ShardedEnsemble over one CPU oracle per member."""

    def __init__(self, params):
        import oracle
        self.orc = [oracle.Oracle(p["NR"], p["NT"], p["NZ"], Re=p["Re"], dt=p["dt"], LZ=p["LZ"], nthreads=1)
                    for p in params]
        self.u = [None] * len(params)

    def set_state(self, m, u):
        self.u[m] = [a.copy() for a in u]

    def step(self, nsteps, check=False):
        import numpy as np
        it = np.zeros((nsteps, len(self.orc)), np.int32)
        for m, o in enumerate(self.orc):
            self.u[m], it[:, m], _ = o.step(self.u[m], nsteps)
        return it

    def get_state(self, m):
        return [a.copy() for a in self.u[m]]

    def friction(self, m):
        return self.orc[m].friction(self.u[m][2])


def _shard_params():
    NR, NT, NZ, Re, dt, LZ = SHARD_CFG
    return [dict(NR=NR, NT=NT, NZ=NZ, Re=Re + 100.0 * m, dt=dt, LZ=LZ) for m in range(SHARD_N)]


def _shard_field(m):
    from nspipe_gb300.initfield import seeded_field
    NR, NT, NZ, _, _, LZ = SHARD_CFG
    return seeded_field(NR, NT, NZ, LZ, 0.05 * (1 + 0.1 * m), 700 + m)


def _sharded_run(rank, world):
    from nspipe_gb300.ensemble import ShardedEnsemble
    ens = ShardedEnsemble(_shard_params(), rank, world, OracleStepper)
    ens.set_states(_shard_field)
    it = ens.step(SHARD_STEPS)
    return ens.gather_iters(it), ens.gather_friction(), ens.gather_states(), (ens.lo, ens.hi)


def _stepping_worker(rank, world, port, q):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "nspipe-gpu_gb300"), os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from test_ensemble_shard import _sharded_run as run
    res = run(rank, world)
    dist.destroy_process_group()
    q.put((rank, res))


def test_gloo_two_ranks_step_their_shards_like_one_rank(oracle_lib):
    import numpy as np
    single_it, single_fr, single_u, span = _sharded_run(0, 1)  # no process group: one rank owns all
    assert span == (0, SHARD_N) and single_it.shape == (SHARD_STEPS, SHARD_N)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port, world = _free_port(), 2
    procs = [ctx.Process(target=_stepping_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [res[r][3] for r in range(world)] == [(0, 3), (3, 5)]
    for r in range(world):
        it, fr, u, _ = res[r]
        assert np.array_equal(it, single_it)
        assert fr == single_fr
        assert len(u) == SHARD_N
        for m in range(SHARD_N):
            for c in range(3):
                assert np.array_equal(u[m][c], single_u[m][c]), (r, m, c)
