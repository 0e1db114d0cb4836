"""Multi-GPU layout of the FX path: replicas, no data-path collective.

A correlation job (inputs x segments x channels) runs whole on one GPU; the
reference's own parallelism is the same -- independent tasks per SPE with no
exchange between them (TaskDispatcher, cellspe-tasklib.cpp).  N GPUs run N
independent jobs: in the benchmark, the same configuration on a different
seeded input per rank (another subband of the array), so the work per GPU is
fixed as N grows (weak scaling).  The only cross-rank traffic is the timing
reduction: every rank's elapsed time, maximised over ranks, divides the
samples that all ranks processed.
"""
from __future__ import annotations


def job_seed(rank: int, base: int = 4) -> int:
    """Seed of the synthetic input that rank `rank` correlates."""
    return base + 1000 * rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest of every rank's `value` (dist: torch.distributed or None)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gsamples(world: int, samples_per_rank: int, ms: float) -> float:
    """Whole-job rate in G samples/s: all ranks' samples over the slowest rank's time."""
    return world * samples_per_rank / (ms * 1e-3) / 1e9
