"""
Multi-GPU use of the force path: one process per GPU, no data-path
collective.

* A single large system runs as independent replicas (one per rank); the
  whole-job rate is the atoms of all ranks over the slowest rank's time.
* A batch of structures is sharded into contiguous slices of structures, one
  per rank; a fitting loss over the batch needs one sum over ranks of the
  loss and of its gradient (``allreduce_sum``), the only collective.

The process group (NCCL on GPUs, gloo on CPUs) is set up by the caller, e.g.
by torchrun; every function here also works without one (world size 1).
"""

import os

import numpy as np

try:
    import torch
    import torch.distributed as dist
except Exception:  # pragma: no cover
    torch = None
    dist = None


def dist_info():
    """(world size, rank, local rank) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _active():
    return dist is not None and dist.is_available() and dist.is_initialized() and \
        dist.get_world_size() > 1


def _device():
    return torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend() == "nccl" else torch.device("cpu")


def max_over_ranks(x):
    """Largest x over the ranks (e.g. the slowest rank's time)."""
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(values):
    """Element-wise sum of a float64 array over the ranks."""
    a = np.ascontiguousarray(values, dtype=np.float64)
    if not _active():
        return a.copy()
    t = torch.from_numpy(a.copy()).to(_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def replica_rate(units_per_rank, seconds, world_size):
    """Whole-job rate of independent replicas: all ranks' units over the
    slowest rank's time (``seconds`` is that maximum)."""
    return world_size * units_per_rank / seconds


def shard_range(n, rank, world_size):
    """Contiguous slice [lo, hi) of n items for ``rank``; sizes differ by at
    most one, lower ranks take the larger ones."""
    q, r = divmod(n, world_size)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def shard(items, rank, world_size):
    lo, hi = shard_range(len(items), rank, world_size)
    return items[lo:hi]


def sharded_fitting_sums(e, e_target, nat, f, f_target):
    """Unnormalised partial sums of the fitting loss on this rank's
    structures: (sum_s (dE_s/N_s)^2, sum_i |dF_i|^2, structures, atoms).
    After allreduce_sum over ranks, loss = s0 / s2 + w_F s1 / s3."""
    de = (np.asarray(e) - np.asarray(e_target)) / np.asarray(nat, dtype=np.float64)
    df = np.asarray(f) - np.asarray(f_target)
    return np.array([np.sum(de * de), np.sum(df * df), len(de), df.shape[0]],
                    dtype=np.float64)
