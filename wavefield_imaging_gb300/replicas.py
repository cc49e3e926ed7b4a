"""Multi-rank use: shots are independent, so ranks (one process per GPU)
take disjoint subsets of a survey's shots and run them with no collective on
the data path.  The one exchange is at the end of a multi-rank misfit
gradient: the per-rank model gradients (FP64) and misfits are summed once
over the host process group (gloo or NCCL through torch.distributed).
survey_gradient runs that split through the engine's batched gradient."""
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


def survey_gradient(desc, shots, vel, wav, dobs, dist=None, device: int = 0, ckpt_format: int = None):
    """Misfit gradient of a 2D survey over ranks.  Every rank runs the
    batched, checkpointed gradient (awe_batch_gradient) of its shard of the
    shots on its own GPU, then the per-rank model gradients and misfits are
    summed once (reduce_gradient).  desc, shots, vel as for Batch; wav [nt];
    dobs: the shots' observed traces, in the order of `shots`.  Returns
    (dJ/dm on the whole model [n2][n1], float64; J) on every rank."""
    from .engine import CKPT_BFP16, Batch

    rank, world = 0, 1
    if dist is not None and dist.is_initialized():
        rank, world = dist.get_rank(), dist.get_world_size()
    mine = shard(range(len(shots)), rank, world)
    grad = np.zeros((desc.n[1], desc.n[0]), np.float64)
    J = 0.0
    if mine:
        with Batch(desc, [shots[i] for i in mine], device=device) as b:
            b.set_model(vel)
            if desc.fdorder == 8:
                try:  # the column-march kernel where the grid allows it
                    b.select(4, chunk=64)
                except Exception:  # noqa: BLE001 - the default tile kernel stays
                    pass
            grad, J = b.gradient(wav, [dobs[i] for i in mine],
                                 ckpt_format=CKPT_BFP16 if ckpt_format is None else ckpt_format)
    return reduce_gradient(grad, J, dist)
