"""Host logic of runs over several GPUs of one node: one process per GPU (torchrun), no collective on the data
path.  The 128^3 workload runs one replica per rank (weak scaling: per-GPU work fixed); the configuration-5
sweep deals its independent problems out to the ranks.  Whole-job throughput is the units all ranks processed
over the slowest rank's time."""
from __future__ import annotations

import os


def env():
    """(world, rank, local rank) from the launcher's environment (1, 0, 0 without one)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items, rank, world):
    """The items of one rank: every world-th item from its rank on (independent problems, no exchange)."""
    return list(items)[rank::world]


def _reduce(value, op, device):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(value, device="cpu"):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX, device)


def reduce_sum(value, device="cpu"):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM, device)


def whole_job_rate(units, ms, device="cpu"):
    """(units of all ranks, slowest rank's ms, units per second of the whole job)."""
    total = reduce_sum(units, device)
    ms_max = reduce_max(ms, device)
    return total, ms_max, total / (ms_max * 1e-3)
