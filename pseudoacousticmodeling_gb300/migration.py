"""The reference's ``migration`` class (src/Migration.py:35, cpp/Migration.cu)
on the engine: reverse-time migration or, with ``fwi`` set, the FWI gradient,
for all shots in batches, with the source field rebuilt from HBM checkpoints,
saved boundary bands or a random border (the reference's "migration" key).
"""
import numpy as np

from . import preprocess
from .engine import RANDOM_BOUNDARY, laplacian_filter_gpu, smooth_model
from .survey import import_bin, save_bin


class migration:
    def __init__(self, wavefield, parameters, ckpt_interval=None, store=None):
        self.wf = wavefield
        self.pmt = parameters
        self.ckpt_interval = parameters.source_field_interval if ckpt_interval is None else ckpt_interval
        self.store = parameters.ckpt_store if store is None else store

    def loadSeismogram(self, shot):
        """The observed data of a shot.  In FWI mode too: the engine forms the
        residual dobs - dcal itself, where the reference writes it to
        residual_shot_*.bin in objective_function (src/Inversion.py:49-51) and
        reads that file back here (src/Migration.py:102-109)."""
        p = self.pmt
        return import_bin(p.seismogram_file(shot), (p.nt_data, p.Nrec))

    def Mute(self, seismogram, shot):
        """cpp/Migration.cu:86-115."""
        p = self.pmt
        return preprocess.mute(seismogram, p.rec_x, p.rec_z, p.shot_x[shot], p.shot_z[shot], p.dt, p.v0, p.shift,
                               p.window)

    def smoothModels(self):
        """Migration::setModel (cpp/Migration.cu:252-309): slowness smoothing of vp,
        value smoothing of the anisotropy parameters, water layer kept."""
        wf, p = self.wf, self.pmt
        # on the GPU, as the drivers do; the water mask of every field comes
        # from the unsmoothed velocity (cpp/Migration.cu:265-290)
        vp = smooth_model(wf.vp, p.sigma)
        eps = None if wf.epsilon is None else smooth_model(wf.epsilon, p.sigma, parameter=True, water_model=wf.vp)
        dl = None if wf.delta is None else smooth_model(wf.delta, p.sigma, parameter=True, water_model=wf.vp)
        th = None if wf.theta is None else smooth_model(wf.theta, p.sigma, parameter=True, water_model=wf.vp)
        return vp, eps, dl, th

    def SolveBackwardWaveEquation(self, observed=None, smooth=True, normalize="cpp", save=True):
        """Image (or gradient when pmt.fwi) of all shots; observed data default to
        the reference's seismogram files.  Returns (image or gradient, illumination).

        Under a torch.distributed process group each rank migrates its
        contiguous share of the shots (distributed.local_shots); the raw
        images (or gradients) and illuminations of the ranks are summed with
        one all-reduce and normalised on the host, and rank 0 writes the
        files."""
        from .distributed import allreduce_sum, local_shots, world_info
        rank, world = world_info()
        p, wf = self.pmt, self.wf
        e = wf.engine
        if smooth and not p.fwi:
            e.set_models(*self.smoothModels())
        e.rtm_reset()
        if self.ckpt_interval == RANDOM_BOUNDARY:
            e.set_random_boundary(p.dvel, p.ratio)
        multi = bool(p.fwi and getattr(p, "multiparameter", False) and p.approximation in ("VTI", "TTI"))
        if p.approximation in ("VTI", "TTI"):
            e.set_multiparameter(multi)
        B = e.cfg.max_shots
        mine = local_shots(p.Nshot)
        for b0 in range(0, mine.size, B):
            idx = mine[b0:b0 + B]
            if observed is None:
                d = np.stack([self.loadSeismogram(int(s)) for s in idx])
            else:
                d = np.asarray(observed[idx], np.float32)
            if not p.fwi:
                # Migration::Mute of every gather, on the GPU after the upload
                e.set_mute(p.shot_x[idx], p.shot_z[idx], p.rec_x, p.rec_z, p.v0, p.shift, p.window)
                e.rtm(p.sz[idx], p.sx[idx], d, ckpt_interval=self.ckpt_interval, store=self.store)
            else:
                e.fwi_gradient(p.sz[idx], p.sx[idx], d, ckpt_interval=self.ckpt_interval, store=self.store)
        save = save and rank == 0
        if not p.fwi:
            if world == 1:
                image, ilum = e.rtm_result(norm=normalize)
            else:
                raw, ilum = e.rtm_result(norm="none")
                n = raw.size
                tot = allreduce_sum(np.concatenate([raw.ravel(), ilum.ravel()]))
                raw = tot[:n].reshape(raw.shape).astype(np.float32)
                ilum = tot[n:].reshape(raw.shape).astype(np.float32)
                image = preprocess.normalize_image(raw, ilum, normalize)
            if save:
                save_bin(p.image_file(), image)
            return image, ilum
        grad, ilum = e.fwi_result()
        if world > 1:
            n = grad.size
            tot = allreduce_sum(np.concatenate([grad.ravel(), ilum.ravel()]))
            grad = tot[:n].reshape(grad.shape).astype(np.float32)
            ilum = tot[n:].reshape(grad.shape).astype(np.float32)
        norm = ilum + 1e-5 * ilum.max()                       # src/Migration.py:1086
        grad = grad / norm
        if save:
            save_bin(p.gradient_file(), grad)
        if multi:
            # src/Migration.py:1087-1104: the same normalisation and file names
            self.multiparameter_gradients = {}
            for name, gx in zip(("epsilon", "delta", "theta"), e.fwi_multiparameter_result()):
                if gx is None:
                    continue
                if world > 1:
                    gx = allreduce_sum(gx).astype(np.float32)
                self.multiparameter_gradients[name] = gx / norm
                if save:
                    save_bin(p.gradient_file(name), gx / norm)
        return grad, ilum

    def laplacian_filter(self, image):
        """-(d2/dz2 + d2/dx2) of the image (src/Viewdata.py:23-41), on the GPU."""
        return laplacian_filter_gpu(image, self.pmt.dz, self.pmt.dx)
