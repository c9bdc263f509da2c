"""Replica bookkeeping for multi-GPU runs.

The time loop does not shard in this build (one GPU per context, no collectives):
with N ranks, each runs an independent replica of the workload on its own GPU, and
the job's throughput is N * steps / (the slowest rank's time). The only exchange is
that max-reduction of the timings, done on whatever process group the caller has
(NCCL on GPUs, gloo in tests).
"""
import os


def rank_env():
    """(rank, world_size, local_rank) from the torchrun environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base_seed, rank):
    """Seed of a rank's replica: the same workload on every rank unless asked otherwise."""
    return int(base_seed)


def max_over_ranks(values, dist=None, device=None):
    """Element-wise max of a list of floats over all ranks (identity without a group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_throughput(steps_per_rank, max_seconds, world_size):
    """Whole-job steps/s: every rank advanced its own replica steps_per_rank steps."""
    return world_size * steps_per_rank / max_seconds
