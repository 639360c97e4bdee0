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


def world_info():
    """(rank, world size) of the default process group, (0, 1) without one."""
    try:
        import torch.distributed as dist
    except ImportError:
        return 0, 1
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def local_shots(n_shots):
    """Indices of the shots this rank handles: all of them in a single
    process, the rank's contiguous share under a process group."""
    rank, world = world_info()
    return shard(n_shots, rank, world) if world > 1 else np.arange(n_shots)


def allreduce_sum(array, device=None):
    """Sum a numpy array over all ranks of the default process group (float64
    on the wire); the array itself, as float64, in a single process.  The
    device defaults to the backend's (CUDA for NCCL, host for gloo)."""
    a = np.ascontiguousarray(array, np.float64)
    rank, world = world_info()
    if world == 1:
        return a.copy()
    import torch
    import torch.distributed as dist
    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(a).to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
