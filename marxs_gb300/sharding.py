"""Photon sharding across ranks (one process per GPU).

Photons are independent (no cross-row coupling anywhere on the path,
simulator.py:42-49), so a multi-GPU run partitions photons by contiguous
global id ranges and needs no data-path collective.  The Philox streams are
keyed by global photon id (``row_base``), so results do not depend on the
partitioning.  The only collective is the max over ranks of the timings.
"""


def strong_shard(rank, world, n_total):
    """Contiguous [start, stop) of ``n_total`` photons for ``rank``."""
    base, extra = divmod(int(n_total), int(world))
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def weak_shard(rank, n_per_rank):
    """Global id range of rank's photons when every rank traces the same count."""
    start = int(rank) * int(n_per_rank)
    return start, start + int(n_per_rank)


def max_over_ranks(values, dist=None, device=None):
    """Element-wise max of a list of floats over all ranks (identity when
    ``dist`` is None or not initialised)."""
    import torch
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()
