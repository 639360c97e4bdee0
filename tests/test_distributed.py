"""Multi-rank path on CPU: two gloo ranks each take their share of the shots,
compute per-shot partial RTM images with the CPU oracle, and sum them with
one all-reduce; the result equals the single-process sum over all shots."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _case():
    from oracle import oracle as O
    g = O.Grid(nz=14, nx=24, N=10, dz=10.0, dx=10.0, dt=0.001, nt=90, itlag=20, fcut=35.0)
    vp = np.full((g.nz, g.nx), 1800.0, np.float32)
    vp[7:, :] = 2400.0
    m = O.Models.build(g, vp)
    src = O.ricker_cpp(g.nt, g.dt, g.fcut, np.float32(0.1), g.dx, g.dz)
    rx = np.arange(g.N, g.N + g.nx, 2)
    rz = np.full(rx.size, g.N + 2)
    sx = g.N + np.array([3, 8, 13, 18, 21])
    d = np.stack([O.forward_shot(g, m, src, int(x), g.N + 1, rx, rz, dtype=np.float32) for x in sx])
    return O, g, m, src, rx, rz, sx, d


def _partial(indices):
    O, g, m, src, rx, rz, sx, d = _case()
    img = np.zeros((g.nz, g.nx))
    for i in indices:
        a, _ = O.rtm_shot(g, m, src, int(sx[i]), g.N + 1, rx, rz, d[i], dtype=np.float32)
        img += a
    return img


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pseudoacousticmodeling_gb300.distributed import allreduce_sum, shard
    total = allreduce_sum(_partial(shard(5, rank, world)))
    if rank == 0:
        np.save(out, total)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_image_sum(tmp_path):
    out = str(tmp_path / "img.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    want = _partial(range(5))
    assert np.abs(want).max() > 0
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def _partial_gradient(indices):
    """Misfit and exact gradient (expanded grid) of the shots in `indices`,
    from the CPU oracle, against data of a slightly faster model."""
    O, g, m, src, rx, rz, sx, _ = _case()
    vp_obs = np.full((g.nz, g.nx), 1850.0, np.float32)
    vp_obs[7:, :] = 2400.0
    m_obs = O.Models.build(g, vp_obs)
    J, grad = 0.0, np.zeros((g.nz_a, g.nx_a))
    for i in indices:
        dobs = O.forward_shot(g, m_obs, src, int(sx[i]), g.N + 1, rx, rz, dtype=np.float64)
        j, gk = O.misfit_and_exact_gradient(g, m, src, int(sx[i]), g.N + 1, rx, rz, dobs, dtype=np.float64)
        J += j
        grad += gk
    return np.concatenate([[J], grad.ravel()])


def _gradient_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pseudoacousticmodeling_gb300.distributed import allreduce_sum, shard
    total = allreduce_sum(_partial_gradient(shard(5, rank, world)))
    if rank == 0:
        np.save(out, total)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_misfit_and_gradient_sum(tmp_path):
    """The FWI exchange: the misfit (a scalar) and the gradient are summed over
    the ranks' shot shards with one all-reduce, and equal the sum over all
    shots in one process."""
    out = str(tmp_path / "grad.npy")
    mp.spawn(_gradient_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    want = _partial_gradient(range(5))
    assert want[0] > 0 and np.abs(want[1:]).max() > 0
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
