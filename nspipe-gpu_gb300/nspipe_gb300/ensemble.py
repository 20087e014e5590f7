"""Sharding an ensemble of independent pipes across GPUs (one process per GPU).

Members never exchange data, so a multi-GPU run is a partition of the member
index range with no collective on the data path: each rank builds, steps and
samples only its own members, and only host-side results (iteration counts,
scalar diagnostics, and states when they are written out) are gathered.  (The
reference is single-GPU: main.cu:16-17 selects device 0 and one pipe.)
"""


def shard(n_members, world_size, rank):
    """Contiguous, balanced slice [lo, hi) of the member range owned by `rank`."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("rank %d outside world of size %d" % (rank, world_size))
    base, extra = divmod(n_members, world_size)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def gather_scalars(values, group=None):
    """All-gather one list of host scalars per rank (torch.distributed, any backend)."""
    import torch
    dist = _dist()
    if dist is None:
        return [list(values)]
    world = dist.get_world_size(group)
    n = torch.tensor([len(values)], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    width = int(max(s.item() for s in sizes))
    buf = torch.zeros(max(width, 1), dtype=torch.float64)
    buf[: len(values)] = torch.tensor(values, dtype=torch.float64)
    out = [torch.zeros(max(width, 1), dtype=torch.float64) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    return [o[: int(s.item())].tolist() for o, s in zip(out, sizes)]


class ShardedEnsemble:
    """This rank's members of a fixed ensemble.

    params       nsp_params of every member of the ensemble, in global member order
    rank, world  this process's rank and the number of processes (one GPU each)
    make_stepper callable(list of nsp_params) -> stepper for this rank's members;
                 the stepper provides set_state(m, u), step(nsteps, check=False) ->
                 iterations (nsteps, n_local), get_state(m) -> [u_r, u_theta, u_z] and
                 friction(m) -> (u_centre, u_tau).  nspipe_gb300.Stepper is one.

    Stepping is local (no collective); the gather_* methods collect host results in
    global member order on every rank and are the only communication (any
    torch.distributed backend; none when the process group is not initialised).
    """

    def __init__(self, params, rank, world, make_stepper):
        self.n = len(params)
        self.lo, self.hi = shard(self.n, world, rank)
        self.params = list(params)
        self.stepper = make_stepper(self.params[self.lo:self.hi]) if self.hi > self.lo else None

    @property
    def members(self):
        return range(self.lo, self.hi)

    def set_states(self, field):
        """field(m) -> [u_r, u_theta, u_z] of global member m; called for this rank's members only."""
        for m in self.members:
            self.stepper.set_state(m - self.lo, field(m))

    def step(self, nsteps):
        """Advances this rank's members; returns their iteration counts (nsteps, n_local)."""
        import numpy as np
        if self.stepper is None:
            return np.zeros((nsteps, 0), np.int32)
        return self.stepper.step(nsteps, check=False)

    def gather_iters(self, iters):
        """Iteration counts (nsteps, n) of every member from each rank's (nsteps, n_local)."""
        import numpy as np
        nsteps = iters.shape[0]
        parts = gather_scalars([float(x) for x in np.asarray(iters).T.reshape(-1)])
        cols = [np.array(p, dtype=np.int64).reshape(-1, nsteps) for p in parts if len(p)]
        return np.concatenate(cols, axis=0).T.astype(np.int32) if cols else np.zeros((nsteps, 0), np.int32)

    def gather_friction(self):
        """(u_centre, u_tau) of every member, global order."""
        vals = []
        for m in self.members:
            vals += list(self.stepper.friction(m - self.lo))
        parts = gather_scalars(vals)
        flat = [v for p in parts for v in p]
        return [(flat[2 * k], flat[2 * k + 1]) for k in range(len(flat) // 2)]

    def gather_states(self):
        """Every member's state on every rank (host arrays), e.g. to write restart files.
        Not part of a step: the data path of stepping has no collective."""
        local = [self.stepper.get_state(m - self.lo) for m in self.members]
        dist = _dist()
        if dist is None:
            return local
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
        return [u for p in parts for u in p]
