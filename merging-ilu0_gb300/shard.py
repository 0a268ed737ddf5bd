"""Multi-GPU batches: every system is independent, so a batch splits into
contiguous slabs of systems, one per rank (one process per GPU), with no
collective on the data path.  The reference runs on one GPU only; this module
is the host-side partition and gathering around the single-GPU solver.

  slab(nsys, rank, world)        -> (first, count) of a rank's systems
  gather(local, group)           -> the global arrays, concatenated in rank order
  max_over_ranks(value, group)   -> the slowest rank's time (a step ends when every rank's has)

Collectives here are host-side bookkeeping (results, timings), never part of
a solve; they run on whatever torch.distributed group the caller set up
(NCCL between GPUs, gloo on CPU)."""


def slab(nsys, rank, world):
    """Contiguous slab of `nsys` systems for `rank` of `world`: the first nsys % world ranks get one more."""
    if world <= 0 or not 0 <= rank < world or nsys < 0:
        raise ValueError("slab: need 0 <= rank < world and nsys >= 0")
    base, rem = divmod(nsys, world)
    first = rank * base + min(rank, rem)
    return first, base + (1 if rank < rem else 0)


def gather(local, group=None):
    """local: dict of per-system numpy arrays (first axis = this rank's systems).  Returns the same keys with
    every rank's arrays concatenated in rank order (on every rank)."""
    import numpy as np
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, {k: np.asarray(v) for k, v in local.items()}, group=group)
    return {k: np.concatenate([p[k] for p in parts]) for k in local}


def max_over_ranks(value, group=None, device=None):
    """The maximum of a float over the ranks (step times: the job's step ends with its slowest rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
