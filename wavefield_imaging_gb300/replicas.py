"""Multi-rank use: shots are independent, so ranks (one process per GPU)
take disjoint subsets of a survey's shots and run them with no collective on
the data path.  The one exchange is at the end of a multi-rank misfit
gradient: the per-rank model gradients (FP64) and misfits are summed once
over the host process group (gloo or NCCL through torch.distributed)."""
from __future__ import annotations

import numpy as np


def shard(items, rank: int, world: int):
    """The items (shots) of `rank` out of `world`: every world-th one, so
    uneven shot sizes spread across ranks."""
    return list(items)[rank::world]


def reduce_gradient(grad: np.ndarray, misfit: float, dist=None):
    """Sum a rank's model gradient and misfit over all ranks (in place for
    `grad`); returns (grad, misfit).  dist = torch.distributed, initialised, or
    None for a single process."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return grad, misfit
    import torch

    t = torch.from_numpy(np.ascontiguousarray(grad, np.float64))
    m = torch.tensor([misfit], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.SUM)
    grad[...] = t.numpy().reshape(grad.shape)
    return grad, float(m.item())
