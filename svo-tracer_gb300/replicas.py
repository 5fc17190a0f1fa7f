"""Multi-GPU runs of the trace: replicas only.

Rays are independent and the octree is read-only during a frame, so N GPUs run N
independent replicas of the workload (one process per GPU, each with its own
context and tree). The only collectives are a barrier around the timed region and
the maximum of the per-rank timings, and the job's throughput counts the rays of
all replicas.
"""
from __future__ import annotations


def max_over_ranks(values, dist=None, device=None):
    """Element-wise maximum over ranks of a list of floats (returned unchanged
    without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def replica_throughput(world: int, rays_per_step: int, ms_per_step: float) -> float:
    """Whole-job Mrays/s: every rank traces `rays_per_step` rays per step, and the
    job's step takes the slowest rank's time."""
    return world * rays_per_step / (ms_per_step / 1000.0) / 1e6
