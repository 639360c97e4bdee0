"""Several GPUs, one process each: shots are independent, so each rank models,
migrates or differentiates its own share of the shots and the only exchange
is one sum of the images / gradients / misfits after the shot loop
(cpp/Modeling.cu:441 loops shots with no coupling between them).

Works with any torch.distributed backend: NCCL on GPUs, gloo on CPU.
"""
import numpy as np


def shard(n_items, rank, world):
    """Contiguous, balanced share of range(n_items) for `rank` of `world`."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return np.arange(start, start + base + (1 if rank < extra else 0))


def allreduce_sum(array, device="cpu"):
    """Sum a numpy array over all ranks of the default process group (float64
    on the wire, so the total does not depend on the rank count's rounding)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(array, np.float64)).to(device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
