"""The multi-rank path on CPU: two gloo ranks run the product's own loops -
the FWI driver (inversion.fwi, src/Inversion.py:290-411) and the migration
class (src/Migration.py:35) - each on its share of the shots, with one
all-reduce of the sums; the results must equal, bitwise, those of one process
running every shot.

The engine is a host stand-in with the engine's interface (no GPU here):
- for FWI, shot i contributes 0.5 |w_i (vp - vtrue)|^2 with a weight from its
  source column;
- for migration, shot i adds an integer pattern to the image and an integer
  to the illumination.
The batch split is chosen so that each rank runs one batch of the
single-process run, which makes the float64 sums identical operation for
operation."""
import os
import socket
from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


class _ShotEngine:
    """Stand-in for Engine in the FWI loop."""

    def __init__(self, vtrue, max_shots):
        self.vtrue = np.asarray(vtrue, np.float32)
        self.cfg = SimpleNamespace(max_shots=max_shots)
        self.vp = self.vtrue
        self.il = None

    @staticmethod
    def _w(sx):
        return (1.0 + (np.asarray(sx) % 5) / 4.0).astype(np.float64)

    def set_models(self, vp):
        self.vp = np.asarray(vp, np.float32)

    def forward(self, sz, sx):
        w = self._w(sx)
        return (w[:, None, None] * self.vp.reshape(1, 1, -1).astype(np.float64)).astype(np.float32)

    def rtm_reset(self):
        self.il = None

    def misfit_gradient(self, sz, sx, dobs, ckpt_interval=0, store="f32"):
        w = self._w(sx)
        r = w[:, None] * self.vp.reshape(1, -1).astype(np.float64) - np.asarray(dobs, np.float64).reshape(len(w), -1)
        g = (w[:, None] * r).sum(0).reshape(self.vp.shape).astype(np.float32)
        self.il = np.full(self.vp.shape, float(w.sum()), np.float32)
        return 0.5 * float((r * r).sum()), g

    def fwi_result(self):
        return None, self.il


def _fwi_problem():
    rng = np.random.default_rng(11)
    vtrue = rng.uniform(1900.0, 2500.0, (5, 6)).astype(np.float32)
    v0 = np.full_like(vtrue, 2200.0)
    sx = np.array([3, 7, 10, 14], np.int32)
    sz = np.zeros(4, np.int32)
    dobs = _ShotEngine(vtrue, 4).forward(sz, sx)
    return vtrue, v0, sz, sx, dobs


def _run_fwi():
    from pseudoacousticmodeling_gb300.inversion import fwi
    vtrue, v0, sz, sx, dobs = _fwi_problem()
    inv = fwi(_ShotEngine(vtrue, 2), sz, sx, dobs, vmin=1500.0, vmax=3000.0, device="cpu")
    vp = inv.solveFullWaveformInversion(v0, niter=4)
    return vp, np.array(inv.history), np.array([len(inv.batches)])


class _MigEngine:
    """Stand-in for Engine in the migration class: integer images."""

    def __init__(self, nz, nx, max_shots):
        self.cfg = SimpleNamespace(max_shots=max_shots)
        self.pattern = (np.arange(nz * nx).reshape(nz, nx) % 7 - 3).astype(np.float32)
        self.rtm_reset()

    def rtm_reset(self):
        self.img = np.zeros_like(self.pattern)
        self.il = np.zeros_like(self.pattern)

    def set_mute(self, *args):
        pass

    def rtm(self, sz, sx, d, ckpt_interval=0, store="f32"):
        for x in np.asarray(sx):
            self.img += np.float32(int(x) % 3 + 1) * self.pattern
            self.il += np.float32(int(x) % 2 + 1) + np.abs(self.pattern)

    def rtm_result(self, norm="cpp"):
        from pseudoacousticmodeling_gb300 import preprocess
        return preprocess.normalize_image(self.img, self.il, norm), self.il.copy()


def _run_migration():
    from pseudoacousticmodeling_gb300.migration import migration
    nz, nx, ns = 4, 9, 5
    sx = np.array([2, 5, 7, 11, 13], np.int32)
    pmt = SimpleNamespace(fwi=False, approximation="acoustic", Nshot=ns, shot_x=sx * 10.0, shot_z=np.zeros(ns),
                          rec_x=np.arange(3) * 10.0, rec_z=np.zeros(3), v0=1500.0, shift=0.0, window=0.01,
                          sz=np.zeros(ns, np.int32), sx=sx, source_field_interval=0, ckpt_store="f32")
    wf = SimpleNamespace(engine=_MigEngine(nz, nx, 3))
    mig = migration(wf, pmt)
    img, ilum = mig.SolveBackwardWaveEquation(observed=np.zeros((ns, 2, 3), np.float32), smooth=False, save=False)
    return img, ilum


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    vp, hist, nb = _run_fwi()
    img, ilum = _run_migration()
    if rank == 0:
        np.savez(out, vp=vp, hist=hist, nb=nb, img=img, ilum=ilum)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_run_the_product_loops_bitwise(tmp_path):
    out = str(tmp_path / "ranks.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    vp, hist, nb = _run_fwi()
    img, ilum = _run_migration()
    # the single process runs two FWI batches; each rank ran one of them
    assert int(nb[0]) == 2 and int(got["nb"][0]) == 1
    assert hist[-1] < hist[0]                       # the inversion made progress
    assert np.array_equal(got["vp"], vp) and np.array_equal(got["hist"], hist)
    assert np.abs(img).max() > 0
    assert np.array_equal(got["img"], img) and np.array_equal(got["ilum"], ilum)


def test_shard_covers_every_shot_once():
    from pseudoacousticmodeling_gb300.distributed import local_shots, shard
    for n in (1, 5, 64, 127):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert np.array_equal(np.concatenate(parts), np.arange(n))
            assert max(p.size for p in parts) - min(p.size for p in parts) <= 1
    assert np.array_equal(local_shots(7), np.arange(7))      # no process group: every shot
