"""Replica bookkeeping for one independent sampler per GPU.

The sampling path shards by chain (each chain, and each posterior of a
posterior set, is an independent unit), so N GPUs run N replicas with no
collective on the data path.  What the ranks share is bookkeeping: disjoint
chain ids (CmdStan numbers chains id, id + 1, ...: src/cmdstan/command.hpp
:657-688 pass `id` to the service) and the whole-job figures of a timed run
(leapfrogs summed over ranks; device and wall time as the slowest rank's).
"""


def chain_id_base(rank, chains_per_rank, first_id=1):
    """First chain id of a rank's replica: ranks own consecutive id blocks."""
    if rank < 0 or chains_per_rank < 1:
        raise ValueError("rank must be >= 0 and chains_per_rank >= 1")
    return first_id + rank * chains_per_rank


def reduce_job(leapfrogs, device_ms, wall_ms, dist=None, device=None):
    """Whole-job (leapfrogs, device_ms, wall_ms): leapfrogs summed over the
    ranks, times the maximum over the ranks.  `dist` is torch.distributed (or
    None for a single process); `device` is where the reduction tensors live
    ("cuda" under NCCL, None / "cpu" under gloo).  A rank that has gone away
    surfaces here as the collective's error."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(leapfrogs), float(device_ms), float(wall_ms)
    import torch
    tot = torch.tensor([float(leapfrogs)], dtype=torch.float64, device=device)
    mx = torch.tensor([float(device_ms), float(wall_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(tot)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    return float(tot[0]), float(mx[0]), float(mx[1])
