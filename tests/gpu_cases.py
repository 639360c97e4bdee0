"""Seeded synthetic cases shared by the GPU parity tests and smoke()."""
import numpy as np

from oracle import oracle as O


def smooth_field(rng, shape, lo, hi, passes=3):
    f = rng.standard_normal(shape)
    k = np.array([1.0, 2.0, 3.0, 2.0, 1.0])
    k /= k.sum()
    for _ in range(passes):
        for ax in (0, 1):
            f = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), ax, f)
    f = (f - f.min()) / (np.ptp(f) + 1e-30)
    return (lo + (hi - lo) * f).astype(np.float32)


def make_case(approx="acoustic", abc="cerjan", nz=70, nx=150, N=20, nt=260, fcut=30.0, nshots=3, seed=0,
              dx=10.0, dz=10.0, dt=0.001, amp=1.0, sd_off=False):
    """A layered model with smooth anisotropy, `nshots` surface shots and a
    receiver every second column three cells below the top of the interior.

    amp scales the reference wavelet; sd_off sets delta = epsilon, which makes
    the pseudo-acoustic Sd term identically zero."""
    rng = np.random.default_rng(seed)
    vp = np.full((nz, nx), 1600.0, np.float32)
    vp[nz // 3:, :] = 2100.0
    vp[2 * nz // 3:, :] = 2600.0
    vp += smooth_field(rng, (nz, nx), -60.0, 60.0)
    eps = smooth_field(rng, (nz, nx), 0.02, 0.22)
    dl = smooth_field(rng, (nz, nx), 0.0, 0.09)
    th = smooth_field(rng, (nz, nx), -35.0, 35.0)
    tlag = 2.0 * np.sqrt(np.pi) / fcut
    itlag = int(round(tlag / dt))
    g = O.Grid(nz=nz, nx=nx, N=N, dz=dz, dx=dx, dt=dt, nt=nt, itlag=itlag, fcut=fcut, approx=approx, abc=abc)
    sx = (N + np.linspace(6, nx - 7, nshots)).astype(np.int32)
    sz = np.full(nshots, N + 2, np.int32)
    rx = np.arange(N, N + nx, 2).astype(np.int32)
    rz = np.full(rx.size, N + 3, np.int32)
    w = (O.ricker_cpp(nt, dt, fcut, np.float32(tlag), dx, dz) * np.float32(amp)).astype(np.float32)
    if sd_off:
        dl = eps.copy()
    return dict(grid=g, vp=vp, eps=eps, delta=dl, theta=th, sx=sx, sz=sz, rx=rx, rz=rz, wavelet=w)


def engine_for(case, max_shots=None):
    from pseudoacousticmodeling_gb300 import Config, Engine
    g = case["grid"]
    cfg = Config(nz=g.nz, nx=g.nx, n_abc=g.N, dz=g.dz, dx=g.dx, dt=g.dt, nt=g.nt, itlag=g.itlag, fcut=g.fcut,
                 approximation=g.approx, boundary=g.abc,
                 max_shots=max_shots or len(case["sx"]))
    e = Engine(cfg)
    e.set_models(case["vp"], case["eps"], case["delta"], case["theta"])
    e.set_wavelet(case["wavelet"])
    e.set_receivers(case["rz"], case["rx"])
    return e


def oracle_models(case):
    g = case["grid"]
    return O.Models.build(g, case["vp"], case["eps"], case["delta"], case["theta"])


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
