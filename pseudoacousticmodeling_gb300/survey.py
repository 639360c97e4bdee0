"""Job description in the reference's own formats.

``parameters`` reads ``Parameters.json`` and the source/receiver CSV files the
reference uses (cpp/Survey.cpp:20-176, src/survey.py:5-145) and derives the
grid sizes.  The two reference front ends disagree on the rounding of derived
sizes: the C++ one rounds (``std::round``, cpp/Survey.cpp:101-108) and the
Python one truncates (``int()``, src/survey.py:41-44, 131-138), which changes
``itlag`` and ``nt_data`` for some configurations.  ``rounding="cpp"`` (the
default) follows the C++ side; ``rounding="python"`` reproduces the Python
side.  Keys beyond the reference's are optional (``batch``, ``ckpt_interval``,
``ckpt_store``).

Binary files keep the reference's layout and names: raw little-endian float32
models [nz][nx], seismograms [nt_data][Nrec] per shot
(cpp/Modeling.cu:397-419), images [nz][nx] (cpp/Migration.cu:337-357).
"""
import csv
import json
import math
import os

import numpy as np

# Keys the C++ reader requires (cpp/Survey.cpp:45-99); the Python reader needs a subset.
REQUIRED = ["unit", "approximation", "migration", "ABC", "dx", "dz", "dt", "L", "D", "T", "N_abc", "fcut"]
DEFAULTS = {"sigma": 20.0, "dvel": 1000.0, "ratio": 200.0, "shift": 0.1, "window": 0.05, "v0": 1500.0,
            "step": 200, "last_save": 1000, "fwi": False, "niter": 15, "freqs": [], "vmin": 1500.0,
            "vmax": 5000.0, "epsmin": 0.0, "epsmax": 0.3, "deltamin": 0.0, "deltamax": 0.2,
            "thetamin": -90.0, "thetamax": 90.0, "multiparameter": False, "reciprocity": False,
            "mirror": False, "layer2": False, "layer3": False, "gradientmodel": False, "diffractor": False,
            "modelfromvp": False, "waterlayer": False, "idx_water": 0, "snap": False,
            "rec_file": "", "src_file": "", "vpFile": "", "epsilonFile": "", "deltaFile": "", "thetaFile": "",
            "snapshotFolder": "", "seismogramFolder": "", "checkpointFolder": "", "imageFolder": "",
            "modelFolder": "", "estimatedmodelsFolder": "", "gradientsFolder": "",
            "batch": 0, "ckpt_interval": 0, "ckpt_store": "f32"}


def read_csv_geometry(path):
    """CSV with a header and columns index, coordx, coordz (cpp/Survey.cpp:20-38)."""
    xs, zs = [], []
    with open(path, newline="") as f:
        rows = csv.reader(f)
        header = next(rows, None)
        if header is None:
            return np.zeros(0), np.zeros(0)
        cols = [h.strip() for h in header]
        ix = cols.index("coordx") if "coordx" in cols else 1
        iz = cols.index("coordz") if "coordz" in cols else 2
        for r in rows:
            if not r:
                continue
            xs.append(float(r[ix]))
            zs.append(float(r[iz]))
    return np.asarray(xs, np.float64), np.asarray(zs, np.float64)


def write_csv_geometry(path, x, z):
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["index", "coordx", "coordz"])
        for i, (a, b) in enumerate(zip(x, z)):
            w.writerow([i, a, b])


def _cpp_round(v):
    """std::round of a float: halves away from zero."""
    return int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


class parameters:
    """The reference's ``parameters`` / ``Survey`` object (src/survey.py:5,
    cpp/Survey.hpp:6).  Attribute names follow the reference."""

    def __init__(self, parameters_path, rounding="cpp", read_geometry=True):
        if rounding not in ("cpp", "python"):
            raise ValueError("rounding must be 'cpp' or 'python'")
        self.parameters_path = parameters_path
        self.rounding = rounding
        self.readParameters()
        if read_geometry:
            self.readAcquisitionGeometry()

    # ------------------------------------------------------------------ parameters
    def readParameters(self):
        with open(self.parameters_path) as f:
            raw = json.load(f)
        missing = [k for k in REQUIRED if k not in raw]
        if missing:
            raise ValueError(f"{self.parameters_path}: missing required keys {missing}")
        self.parameters = dict(DEFAULTS)
        self.parameters.update(raw)
        for k, v in self.parameters.items():
            setattr(self, k, v)
        if self.approximation not in ("acoustic", "VTI", "TTI"):
            raise ValueError(f"unknown approximation {self.approximation!r}: choose 'acoustic', 'VTI' or 'TTI'")
        if self.ABC not in ("cerjan", "CPML"):
            raise ValueError(f"unknown ABC {self.ABC!r}: choose 'cerjan' or 'CPML'")
        if self.migration not in ("onthefly", "checkpoint", "SB", "RBC"):
            raise ValueError(f"unknown migration method {self.migration!r}: choose 'onthefly', 'checkpoint', 'SB' "
                             "or 'RBC'")
        # source-field strategy of the engine (src/Migration.py:1563-1583): every
        # step stored, checkpoints every ckpt_interval (else `step`) steps,
        # boundary saving (-1) or the random border (-2)
        self.source_field_interval = {"onthefly": 0, "SB": -1, "RBC": -2}.get(
            self.migration, int(self.ckpt_interval) if int(self.ckpt_interval) > 0 else int(self.step))
        base = os.path.dirname(os.path.abspath(self.parameters_path))
        for k in ("rec_file", "src_file", "vpFile", "epsilonFile", "deltaFile", "thetaFile", "snapshotFolder",
                  "seismogramFolder", "checkpointFolder", "imageFolder", "modelFolder", "estimatedmodelsFolder",
                  "gradientsFolder"):
            v = getattr(self, k)
            if v and not os.path.isabs(v):
                setattr(self, k, os.path.normpath(os.path.join(base, v)) + (os.sep if v.endswith("/") else ""))
        self.tlag = 2.0 * math.sqrt(math.pi) / self.fcut
        if self.rounding == "cpp":
            # float arithmetic then std::round (cpp/Survey.cpp:101-108)
            f = np.float32
            tlag = f(2.0) * np.sqrt(f(np.pi), dtype=f) / f(self.fcut)
            self.tlag = float(tlag)
            self.itlag = _cpp_round(float(tlag / f(self.dt)))
            self.nt_data = _cpp_round(float(f(self.T) / f(self.dt))) + 1
            self.nx = _cpp_round(float(f(self.L) / f(self.dx))) + 1
            self.nz = _cpp_round(float(f(self.D) / f(self.dz))) + 1
        else:
            # src/survey.py:38-45
            self.itlag = int(self.tlag / self.dt)
            self.nt_data = int(self.T / self.dt) + 1
            self.nx = int(self.L / self.dx) + 1
            self.nz = int(self.D / self.dz) + 1
        self.nt = self.itlag + self.nt_data
        self.nx_abc = self.nx + 2 * self.N_abc
        self.nz_abc = self.nz + 2 * self.N_abc
        self.x = np.arange(self.nx) * self.dx
        self.z = np.arange(self.nz) * self.dz
        self.t = np.arange(self.nt) * self.dt

    # ------------------------------------------------------------------ geometry
    def readAcquisitionGeometry(self):
        """Receiver and source coordinates to expanded-grid indices
        (cpp/Survey.cpp:128-176): round(coord/d) + N_abc (C++) or int() (Python),
        with the reference's reciprocity swap and mirror shift."""
        self.rec_x, self.rec_z = read_csv_geometry(self.rec_file)
        self.shot_x, self.shot_z = read_csv_geometry(self.src_file)
        if self.reciprocity:
            self.shot_x, self.rec_x = self.rec_x.copy(), self.shot_x.copy()
            self.shot_z, self.rec_z = self.rec_z.copy(), self.shot_z.copy()
        self.Nrec = len(self.rec_x)
        self.Nshot = len(self.shot_x)
        self.rx, self.rz = self._to_grid(self.rec_x, self.dx), self._to_grid(self.rec_z, self.dz)
        self.sx, self.sz = self._to_grid(self.shot_x, self.dx), self._to_grid(self.shot_z, self.dz)
        if self.mirror:
            self.rz = self.rz - int(self.idx_water)
            self.sz = self.sz - int(self.idx_water)

    def _to_grid(self, c, d):
        if self.rounding == "cpp":
            f = np.float32
            return np.asarray([_cpp_round(float(f(v) / f(d))) for v in c], np.int32) + self.N_abc
        return (np.asarray(c / d).astype(np.int32) + self.N_abc).astype(np.int32)

    # ------------------------------------------------------------------ files
    def seismogram_file(self, shot):
        """cpp/Modeling.cu:400 naming (fcut with one decimal)."""
        return os.path.join(self.seismogramFolder,
                            f"seismogram_shot_{shot + 1}_Nt{self.nt_data}_Nrec{self.Nrec}_fcut{self.fcut:.1f}.bin")

    def residual_file(self, shot):
        """src/Inversion.py:285-288 naming."""
        return os.path.join(self.seismogramFolder, f"residual_shot_{shot + 1}_Nt{self.nt_data}_Nrec{self.Nrec}.bin")

    def image_file(self):
        """cpp/Migration.cu:338 naming."""
        return os.path.join(self.imageFolder, f"image_{self.approximation}_Nx{self.nx}_Nz{self.nz}.bin")

    def gradient_file(self, parameter=None):
        """src/Migration.py:1095-1104 naming: gradient_..., or epsilon_gradient_...,
        delta_gradient_..., theta_gradient_... for the multiparameter ones."""
        prefix = "" if parameter is None else f"{parameter}_"
        return os.path.join(self.gradientsFolder,
                            f"{prefix}gradient_{self.approximation}_Nx{self.nx}_Nz{self.nz}.bin")

    def lag_steps(self, fcut):
        """itlag of a cutoff frequency: tlag = 2 sqrt(pi)/fcut over dt, rounded
        like cpp/Survey.cpp:101-102 (std::round) or src/survey.py:41 (int)."""
        if self.rounding == "cpp":
            f = np.float32
            tlag = f(2.0) * np.sqrt(f(np.pi), dtype=f) / f(fcut)
            return _cpp_round(float(tlag / f(self.dt)))
        return int(2.0 * math.sqrt(math.pi) / fcut / self.dt)

    def engine_config(self, max_shots=None, fcut=None):
        """Engine configuration of this job; `fcut` overrides the cutoff
        frequency, and with it the wavelet lag and the step count, as
        fwi.adjustfmax does between frequency bands (src/Inversion.py:285-296)."""
        from .engine import Config
        fc = float(self.fcut if fcut is None else fcut)
        itlag = self.itlag if fcut is None else self.lag_steps(fc)
        return Config(nz=self.nz, nx=self.nx, n_abc=self.N_abc, dz=float(self.dz), dx=float(self.dx),
                      dt=float(self.dt), nt=itlag + self.nt_data, itlag=itlag, fcut=fc,
                      approximation=self.approximation, boundary=self.ABC,
                      max_shots=max_shots or (self.batch or self.Nshot))


def import_bin(path, shape):
    """Raw float32 file (cpp/Modeling.cu:102-109); errors like the reference's
    std::invalid_argument when the file is missing, and on short files."""
    if not os.path.exists(path):
        raise ValueError(f"Could not open file {path!r}. Please verify the file path.")
    a = np.fromfile(path, dtype=np.float32)
    n = int(np.prod(shape))
    if a.size < n:
        raise ValueError(f"{path!r} holds {a.size} floats, {n} expected for shape {tuple(shape)}")
    return a[:n].reshape(shape)


def save_bin(path, array):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.ascontiguousarray(array, np.float32).tofile(path)
