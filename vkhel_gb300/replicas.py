"""Independent replicas across ranks (one process per GPU).

Every limb product is independent, so N GPUs run N replicas of the workload
with no collective on the data path.  The only cross-rank steps are the
barrier around the timed region and the reduction of the result: the job
time is the slowest rank's time and the throughput counts every rank's units.
"""
import torch.distributed as dist


def rank_seed(base, rank):
    """Each rank draws its own operands."""
    return base + 1000 * rank


def shard(items, rank, world):
    """Round-robin share of `items` for `rank` (for workloads given as a list)."""
    return items[rank::world]


def aggregate(local_seconds, local_units):
    """(total units, max seconds, units per second over all ranks).

    Without an initialised process group this is the single-rank result.
    """
    if not (dist.is_available() and dist.is_initialized()):
        return local_units, local_seconds, local_units / local_seconds
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return u.item(), t.item(), u.item() / t.item()
