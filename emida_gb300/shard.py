"""Several GPUs: ROI pairs are independent, so patterns are sharded across
ranks (one process per GPU) with no collective on the data path.  The only
collectives are the timing barrier and the max of the per-rank times, from
which the whole-job throughput is computed."""
import os


def dist_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def pattern_shard(n_patterns, rank, world):
    """Contiguous [first, last) patterns of `rank` when n_patterns are split
    over `world` ranks; the first n_patterns % world ranks get one more."""
    base, extra = divmod(n_patterns, world)
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def max_over_ranks(value, dist=None, device=None):
    """The maximum of a per-rank float (the slowest rank's time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, max_seconds, world):
    """Units per second of the whole job: every rank processed units_per_rank
    (weak scaling) in at most max_seconds."""
    return world * units_per_rank / max_seconds
