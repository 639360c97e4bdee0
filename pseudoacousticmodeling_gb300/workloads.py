"""Seeded synthetic inputs with the shapes of the benchmark configurations.

There is no public dataset for this path; every model here is generated from
a fixed seed with the sizes and value ranges of the configuration it stands in
for.  Sizes follow the Survey arithmetic of cpp/Survey.cpp:101-108
(itlag = round(tlag/dt), nt_data = round(T/dt) + 1, n_abc = n + 2 N).
"""
import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Workload:
    name: str
    nz: int
    nx: int
    dz: float
    dx: float
    dt: float
    nt_data: int
    fcut: float
    n_abc: int
    approximation: str
    boundary: str
    shots: int
    vp: np.ndarray
    eps: np.ndarray = None
    delta: np.ndarray = None
    theta: np.ndarray = None
    sx: np.ndarray = None      # expanded-grid source columns
    sz: np.ndarray = None
    rx: np.ndarray = None      # expanded-grid receiver columns (shared by all shots)
    rz: np.ndarray = None

    @property
    def itlag(self):
        tlag = 2.0 * math.sqrt(math.pi) / self.fcut
        return int(round(tlag / self.dt))

    @property
    def nt(self):
        return self.itlag + self.nt_data

    @property
    def cells_expanded(self):
        return (self.nz + 2 * self.n_abc) * (self.nx + 2 * self.n_abc)

    def config(self, max_shots=None):
        from .engine import Config
        return Config(nz=self.nz, nx=self.nx, n_abc=self.n_abc, dz=self.dz, dx=self.dx, dt=self.dt, nt=self.nt,
                      itlag=self.itlag, fcut=self.fcut, approximation=self.approximation, boundary=self.boundary,
                      max_shots=max_shots or self.shots)


def smooth_random_field(rng, shape, lo, hi, sigma_cells):
    """Gaussian-smoothed white noise rescaled to [lo, hi] (separable FFT filter)."""
    f = rng.standard_normal(shape)
    for ax, n in enumerate(shape):
        k = np.fft.rfftfreq(n)
        filt = np.exp(-2.0 * (math.pi * sigma_cells * k) ** 2)
        f = np.fft.irfft(np.fft.rfft(f, axis=ax) * filt.reshape([-1 if a == ax else 1 for a in range(2)]), n=n, axis=ax)
    f = (f - f.min()) / (np.ptp(f) + 1e-30)
    return (lo + (hi - lo) * f).astype(np.float32)


def batched_vti(shots=128, seed=2, scale=1.0):
    """Batched VTI modelling with CPML: 801 x 2001 at 10 m, six layers
    1500-4000 m/s at seed-drawn depths, epsilon in [0, 0.25] and delta in
    [0, 0.1] as smooth random fields, 12 Hz Ricker, dt 0.8 ms, 4000 samples,
    sources every 15 grid points at z = 10 m, 2001 receivers at z = 10 m.
    `scale` < 1 shrinks the grid and the sample count for tests."""
    rng = np.random.default_rng(seed)
    nz, nx = int(round(800 * scale)) + 1, int(round(2000 * scale)) + 1
    nt_data = max(int(round(4000 * scale)), 50)
    dz = dx = 10.0
    depths = np.sort(rng.uniform(0.08, 0.92, 5)) * (nz - 1) * dz
    vels = np.linspace(1500.0, 4000.0, 6)
    z = np.arange(nz)[:, None] * dz
    vp = np.full((nz, nx), vels[0], np.float32)
    for d, v in zip(depths, vels[1:]):
        vp = np.where(z >= d, np.float32(v), vp)
    eps = smooth_random_field(rng, (nz, nx), 0.0, 0.25, 25.0)
    dl = smooth_random_field(rng, (nz, nx), 0.0, 0.1, 25.0)
    N = 50
    i = np.arange(shots)
    sx = (np.round(15.0 * dx * i / dx).astype(np.int64) % nx + N).astype(np.int32)
    sz = np.full(shots, int(round(10.0 / dz)) + N, np.int32)
    rx = (np.arange(nx) + N).astype(np.int32)
    rz = np.full(nx, int(round(10.0 / dz)) + N, np.int32)
    return Workload("batched VTI pseudo-acoustic modelling, CPML", nz, nx, dz, dx, 0.0008, nt_data, 12.0, N, "VTI",
                    "CPML", shots, vp, eps, dl, None, sx, sz, rx, rz)


def plain_acoustic():
    """Plain 2-D acoustic modelling: 201 x 401 at 10 m, two layers
    (1500 above z = 1000 m, 2500 below), 15 Hz Ricker at (2000 m, 20 m), 401
    receivers at z = 20 m, dt 1 ms, 2001 samples, 50-cell Cerjan border."""
    nz, nx, h = 201, 401, 10.0
    vp = np.full((nz, nx), 1500.0, np.float32)
    vp[int(round(1000.0 / h)):, :] = 2500.0
    N = 50
    rx = (np.arange(nx) + N).astype(np.int32)
    rz = np.full(nx, int(round(20.0 / h)) + N, np.int32)
    return Workload("plain acoustic modelling, Cerjan", nz, nx, h, h, 0.001, 2001, 15.0, N, "acoustic", "cerjan", 1,
                    vp, None, None, None, np.array([int(round(2000.0 / h)) + N], np.int32),
                    np.array([int(round(20.0 / h)) + N], np.int32), rx, rz)


def batched_tti(shots=64, seed=3, scale=1.0):
    """Batched TTI modelling with CPML: 1201 x 3001 at 8 m, dipping layers
    1500-4500 m/s, epsilon in [0, 0.3], delta in [0, 0.15], tilt in
    [-40, 40] degrees following the dip, 10 Hz Ricker, dt 0.6 ms, 6000 samples."""
    rng = np.random.default_rng(seed)
    nz, nx = int(round(1200 * scale)) + 1, int(round(3000 * scale)) + 1
    nt_data = max(int(round(6000 * scale)), 50)
    h = 8.0
    dip = np.deg2rad(rng.uniform(-20.0, 20.0))
    x = np.arange(nx)[None, :] * h
    z = np.arange(nz)[:, None] * h
    zz = z - np.tan(dip) * (x - x.mean())
    depths = np.sort(rng.uniform(0.1, 0.9, 6)) * (nz - 1) * h
    vels = np.linspace(1500.0, 4500.0, 7)
    vp = np.full((nz, nx), vels[0], np.float32)
    for d, v in zip(depths, vels[1:]):
        vp = np.where(zz >= d, np.float32(v), vp)
    eps = smooth_random_field(rng, (nz, nx), 0.0, 0.3, 25.0)
    dl = smooth_random_field(rng, (nz, nx), 0.0, 0.15, 25.0)
    theta = np.clip(np.full((nz, nx), np.rad2deg(dip), np.float32)
                    + smooth_random_field(rng, (nz, nx), -20.0, 20.0, 40.0), -40.0, 40.0).astype(np.float32)
    N = 50
    sx = (np.linspace(0, nx - 1, shots).round().astype(np.int32) + N).astype(np.int32)
    sz = np.full(shots, 1 + N, np.int32)
    rx = (np.arange(nx) + N).astype(np.int32)
    rz = np.full(nx, 1 + N, np.int32)
    return Workload("batched TTI pseudo-acoustic modelling, CPML", nz, nx, h, h, 0.0006, nt_data, 10.0, N, "TTI",
                    "CPML", shots, vp, eps, dl, theta, sx, sz, rx, rz)


def bandpass(w, dt, f_lo, f_hi, taper=1.0):
    """Zero-phase band-pass by an FFT mask with cosine tapers `taper` Hz wide
    at both corners (the 5-10 Hz source band of the gradient workload)."""
    n = w.size
    f = np.fft.rfftfreq(n, dt)
    m = np.zeros_like(f)
    m[(f >= f_lo) & (f <= f_hi)] = 1.0
    lo = (f >= f_lo - taper) & (f < f_lo)
    m[lo] = 0.5 - 0.5 * np.cos(np.pi * (f[lo] - (f_lo - taper)) / taper)
    hi = (f > f_hi) & (f <= f_hi + taper)
    m[hi] = 0.5 + 0.5 * np.cos(np.pi * (f[hi] - f_hi) / taper)
    return np.fft.irfft(np.fft.rfft(w.astype(np.float64)) * m, n=n).astype(np.float32)


def fwi_acoustic(shots=64, seed=5, scale=1.0):
    """Acoustic FWI gradient: 501 x 1701 at 10 m, true model = five layers
    1500-3500 m/s plus 20 seed-placed Gaussian anomalies of +-300 m/s (radius
    80-200 m), starting model = the true model smoothed with a 250 m Gaussian,
    8 Hz Ricker band-passed to 5-10 Hz, dt 1 ms, 3000 samples, 50-cell Cerjan
    border, sources evenly spread at z = 10 m, one receiver per surface column
    at z = 10 m.  Returns (workload with the starting model, true vp, wavelet)."""
    from . import preprocess
    rng = np.random.default_rng(seed)
    nz, nx = int(round(500 * scale)) + 1, int(round(1700 * scale)) + 1
    nt_data = max(int(round(3000 * scale)), 50)
    h = 10.0
    z = np.arange(nz)[:, None] * h
    x = np.arange(nx)[None, :] * h
    depths = np.sort(rng.uniform(0.15, 0.85, 4)) * (nz - 1) * h
    vels = np.linspace(1500.0, 3500.0, 5)
    vtrue = np.full((nz, nx), vels[0])
    for d, v in zip(depths, vels[1:]):
        vtrue = np.where(z >= d, v, vtrue)
    for _ in range(20):
        cz, cx = rng.uniform(0.2, 0.95) * (nz - 1) * h, rng.uniform(0.05, 0.95) * (nx - 1) * h
        r = rng.uniform(80.0, 200.0) * max(scale, 0.25)
        vtrue = vtrue + rng.choice([-300.0, 300.0]) * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * r * r))
    vtrue = vtrue.astype(np.float32)
    sig = 250.0 / h
    vstart = vtrue.astype(np.float64)
    for ax, n in enumerate(vstart.shape):
        # edge-padded FFT smoothing so the borders keep their velocity
        pad = int(4 * sig)
        vp = np.pad(vstart, [(pad, pad) if a == ax else (0, 0) for a in range(2)], mode="edge")
        m = vp.shape[ax]
        k = np.fft.rfftfreq(m)
        filt = np.exp(-2.0 * (math.pi * sig * k) ** 2)
        vp = np.fft.irfft(np.fft.rfft(vp, axis=ax) * filt.reshape([-1 if a == ax else 1 for a in range(2)]), n=m,
                          axis=ax)
        vstart = np.take(vp, np.arange(pad, pad + n), axis=ax)
    vstart = vstart.astype(np.float32)
    N = 50
    sx = (np.linspace(0, nx - 1, shots).round().astype(np.int32) + N).astype(np.int32)
    sz = np.full(shots, int(round(10.0 / h)) + N, np.int32)
    rx = (np.arange(nx) + N).astype(np.int32)
    rz = np.full(nx, int(round(10.0 / h)) + N, np.int32)
    wl = Workload("acoustic FWI gradient, Cerjan", nz, nx, h, h, 0.001, nt_data, 8.0, N, "acoustic", "cerjan",
                  shots, vstart, None, None, None, sx, sz, rx, rz)
    w = preprocess.ricker(wl.nt, wl.dt, wl.fcut, h, h)
    w = bandpass(w, wl.dt, 5.0, 10.0)
    return wl, vtrue, w


def rtm_acoustic(shots=16, seed=7, scale=1.0, first_shot=0):
    """Acoustic RTM: 1001 x 4001 at 5 m, smoothed layered background
    1500-3500 m/s plus seed-placed Gaussian reflectors and a fault-offset
    interface, 20 Hz Ricker, dt 0.4 ms, 8000 samples, 50-cell Cerjan border.
    200 split-spread shots along the surface at z = 10 m (this returns
    `shots` of them from `first_shot`), each with 1601 receivers every 2 cells
    centred on its source (clamped to the grid): per-shot receiver spreads.
    Returns (workload with the migration velocity, true vp)."""
    rng = np.random.default_rng(seed)
    nz, nx = int(round(1000 * scale)) + 1, int(round(4000 * scale)) + 1
    nt_data = max(int(round(8000 * scale)), 50)
    h = 5.0
    z = np.arange(nz)[:, None] * h
    x = np.arange(nx)[None, :] * h
    depths = np.sort(rng.uniform(0.15, 0.85, 4)) * (nz - 1) * h
    throw = rng.uniform(40.0, 120.0)
    fault_x = rng.uniform(0.3, 0.7) * (nx - 1) * h
    vels = np.linspace(1500.0, 3500.0, 5)
    vtrue = np.full((nz, nx), vels[0])
    for i, (d, v) in enumerate(zip(depths, vels[1:])):
        dd = d + (throw if i >= 2 else 0.0) * (x > fault_x)          # the deeper interfaces are offset
        vtrue = np.where(z >= dd, v, vtrue)
    for _ in range(12):
        cz, cx = rng.uniform(0.2, 0.9) * (nz - 1) * h, rng.uniform(0.05, 0.95) * (nx - 1) * h
        r = rng.uniform(15.0, 40.0) * max(scale, 0.25)
        vtrue = vtrue + rng.choice([-250.0, 250.0]) * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * r * r))
    vtrue = vtrue.astype(np.float32)
    # migration velocity: the layered background smoothed over 100 m (no reflectors)
    vmig = vtrue.astype(np.float64)
    sig = 100.0 / h
    for ax, n in enumerate(vmig.shape):
        pad = int(4 * sig)
        vp = np.pad(vmig, [(pad, pad) if a == ax else (0, 0) for a in range(2)], mode="edge")
        m = vp.shape[ax]
        k = np.fft.rfftfreq(m)
        filt = np.exp(-2.0 * (math.pi * sig * k) ** 2)
        vp = np.fft.irfft(np.fft.rfft(vp, axis=ax) * filt.reshape([-1 if a == ax else 1 for a in range(2)]), n=m,
                          axis=ax)
        vmig = np.take(vp, np.arange(pad, pad + n), axis=ax)
    vmig = vmig.astype(np.float32)
    N = 50
    all_sx = np.linspace(0, nx - 1, 200).round().astype(np.int64)
    sel = all_sx[first_shot:first_shot + shots]
    nrec = min(1601, nx)
    half = (nrec - 1)                     # receivers every 2 cells on either side: 2 * 800 cells
    rx = np.empty((sel.size, nrec), np.int32)
    for b, s in enumerate(sel):
        lo = int(np.clip(s - half, 0, max(nx - 1 - 2 * (nrec - 1), 0)))
        rx[b] = np.minimum(lo + 2 * np.arange(nrec), nx - 1) + N
    rz = np.full_like(rx, int(round(10.0 / h)) + N)
    sx = (sel + N).astype(np.int32)
    sz = np.full(sel.size, int(round(10.0 / h)) + N, np.int32)
    wl = Workload("acoustic RTM, Cerjan, split-spread", nz, nx, h, h, 0.0004, nt_data, 20.0, N, "acoustic",
                  "cerjan", int(sel.size), vmig, None, None, None, sx, sz, rx, rz)
    return wl, vtrue
