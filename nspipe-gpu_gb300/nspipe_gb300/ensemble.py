"""Sharding an ensemble of independent pipes across GPUs (one process per GPU).

Members never exchange data, so a multi-GPU run is a partition of the member
index range with no collective on the data path; only scalar diagnostics are
gathered on the host.  (The reference is single-GPU: main.cu:16-17 selects
device 0 and one pipe.)
"""


def shard(n_members, world_size, rank):
    """Contiguous, balanced slice [lo, hi) of the member range owned by `rank`."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("rank %d outside world of size %d" % (rank, world_size))
    base, extra = divmod(n_members, world_size)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def gather_scalars(values, group=None):
    """All-gather one list of host scalars per rank (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return [list(values)]
    world = dist.get_world_size(group)
    n = torch.tensor([len(values)], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    width = int(max(s.item() for s in sizes))
    buf = torch.zeros(width, dtype=torch.float64)
    buf[: len(values)] = torch.tensor(values, dtype=torch.float64)
    out = [torch.zeros(width, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    return [o[: int(s.item())].tolist() for o, s in zip(out, sizes)]
