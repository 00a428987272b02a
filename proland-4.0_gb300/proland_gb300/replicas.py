"""Replicas across GPUs: the tile path shards by quadtree subtree with no
exchange step, so N GPUs run N independent frames (weak scaling) and only the
timing is combined: each rank's step time, the maximum over ranks, and the
whole-job throughput N x tiles / max time."""
import torch


def max_over_ranks(value, dist=None, device="cpu"):
    """Maximum of a per-rank float over the process group (the rank itself if
    there is no group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, ms_per_step_max, world):
    """Units per second of the whole job: every rank did `units_per_rank` units
    in at most `ms_per_step_max` milliseconds."""
    return world * units_per_rank / (ms_per_step_max / 1000.0)


def rank_seed(seed, rank):
    """Each replica produces a different frame of the same shape."""
    return seed + 7919 * rank
