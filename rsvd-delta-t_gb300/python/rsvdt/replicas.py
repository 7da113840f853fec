"""Replicas across GPUs (one process per GPU, launched by torchrun).

The time-stepping path shards naturally by independent problems (or test
vectors): every rank solves its own replica with its own seeded sketch and
no data-path collective. The only cross-rank steps are the barrier before
the timed region and the maximum of the ranks' times after it, from which
the whole-job throughput is formed (weak scaling: per-rank work fixed)."""
from __future__ import annotations


def rank_seed(base: int, rank: int) -> int:
    """Sketch seed of a replica: distinct per rank, reproducible."""
    return base + rank


def max_over_ranks(ms: float, dist=None, device: str = "cpu") -> float:
    """The largest of the ranks' timed-region durations (every rank
    receives it); `dist` is torch.distributed or None for one process."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(ms)
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms_max: float, world: int) -> float:
    """Units per second of the whole job: every rank processed
    units_per_rank in at most ms_max milliseconds."""
    return world * units_per_rank / (ms_max * 1e-3)
