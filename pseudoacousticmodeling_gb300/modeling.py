"""The reference's ``wavefield`` class (src/Modeling2D.py:23-475) on the engine.

Same method names and file conventions; the time loop runs on the GPU, all
shots of a batch at once.  ``forward_step(k)`` keeps the reference's per-step
loop available (it advances every shot of the current batch by one step).
"""
import time

import numpy as np

from . import preprocess
from .engine import Engine
from .survey import import_bin, save_bin


class wavefield:
    def __init__(self, parameters, device=0, wavelet="cpp"):
        self.pmt = parameters
        self.device = device
        self.wavelet = wavelet
        self.engine = None

    # ---------------------------------------------------------------- inputs
    def createSourceWavelet(self):
        p = self.pmt
        if self.wavelet == "cpp":        # cpp/Modeling.cu:84-100
            self.source = preprocess.ricker(p.nt, p.dt, p.fcut, p.dx, p.dz)
        else:                            # src/utils.py:21-28 with src/Modeling2D.py:30
            self.source = preprocess.ricker_half_derivative(p.nt, p.dt, p.fcut, p.dx, p.dz)
        print(f"info: Ricker Source wavelet created: {p.nt} samples")

    def ImportModel(self, filename):
        data = import_bin(filename, (self.pmt.nz, self.pmt.nx))
        print(f"info: Imported: {filename}")
        return data

    def ExpandModel(self, model_data):
        return np.pad(np.asarray(model_data, np.float32), self.pmt.N_abc, mode="edge")

    def loadModels(self):
        p = self.pmt
        self.vp = self.ImportModel(p.vpFile)
        self.epsilon = self.delta = self.theta = None
        if p.approximation in ("VTI", "TTI"):
            self.epsilon = self.ImportModel(p.epsilonFile)
            self.delta = self.ImportModel(p.deltaFile)
        if p.approximation == "TTI":
            self.theta = self.ImportModel(p.thetaFile)      # degrees, converted inside the engine
        print(f"info: Models loaded: {p.nx}x{p.nz}")

    def initializeWavefields(self, max_shots=None):
        p = self.pmt
        if self.engine is None:
            self.engine = Engine(p.engine_config(max_shots), device=self.device)
        if not hasattr(self, "source"):
            self.createSourceWavelet()
        if self.wavelet != "cpp":
            # the engine's own wavelet is the C++ one, computed by the same host
            # code as the reference's (cpp/Modeling.cu:84-100); replace it only
            # for the Python modeller's filtered wavelet
            self.engine.set_wavelet(self.source)
        self.engine.set_receivers(p.rz, p.rx)

    def setModels(self, vp=None, epsilon=None, delta=None, theta=None):
        if vp is not None:
            self.vp = vp
        if epsilon is not None:
            self.epsilon = epsilon
        if delta is not None:
            self.delta = delta
        if theta is not None:
            self.theta = theta
        self.engine.set_models(self.vp, self.epsilon, self.delta, self.theta)

    def checkDispersionAndStability(self):
        ok, dt_lim, dx_lim = self.engine.check_stability()
        p = self.pmt
        print("info: Dispersion and stability check")
        print(f"info: Current dx: {p.dx:.2f} m, dz: {p.dz:.2f} m, dt: {p.dt:.5f} s")
        print(f"info: Critical dx for dispersion: {dx_lim:.2f} m")
        print(f"info: Critical dt for stability: {dt_lim:.5f} s")
        print("info: Dispersion and stability conditions satisfied." if ok else
              "WARNING: Dispersion or stability conditions not satisfied.")
        return ok

    # ---------------------------------------------------------------- stepping
    def begin_shots(self, shots):
        """Reset the fields of the given shot indices (one batch) and inject step 0."""
        self._batch = list(shots)
        self.engine.begin(self.pmt.sz[self._batch], self.pmt.sx[self._batch])

    def forward_step(self, k):
        """One time step of the current batch (src/Modeling2D.py:335-386)."""
        self.engine.step(k)

    def seismograms(self):
        return self.engine.read_seismograms()

    def save_seismogram(self, shot, seismogram):
        path = self.pmt.seismogram_file(shot)
        save_bin(path, seismogram)
        print(f"info: Seismogram saved to {path}")

    def SolveWaveEquation(self, save=True):
        """All shots, batched (src/Modeling2D.py:469-475); returns [Nshot][nt_data][Nrec]."""
        p = self.pmt
        if self.engine is None:
            self.initializeWavefields()
            self.setModels()
        t0 = time.time()
        B = self.engine.cfg.max_shots
        out = np.empty((p.Nshot, p.nt_data, p.Nrec), np.float32)
        for b0 in range(0, p.Nshot, B):
            idx = np.arange(b0, min(b0 + B, p.Nshot))
            out[idx] = self.engine.forward(p.sz[idx], p.sx[idx])
            if save:
                for s in idx:
                    self.save_seismogram(int(s), out[s])
        print(f"info: {p.Nshot} shots completed in {time.time() - t0:.2f} seconds")
        return out
