"""The reference's own code, run unmodified (TEST INFRASTRUCTURE).

``oracle/build.py`` compiles, wherever the reference sources are present:
- cpp/Modeling.cu and cpp/Migration.cu into cubins (``oracle/_ref/*.cubin``),
  which ``oracle/ref_harness.cpp`` loads through the CUDA driver API to repeat
  the reference's modelling shot loop (cpp/Modeling.cu:433-479: ``forward``)
  and its on-the-fly migration (cpp/Migration.cu:359-397: ``rtm``); the host
  preparation (padding, radians, wavelet, Cerjan vector) comes from the
  oracle's restatements of cpp/Modeling.cu:84-182;
- the same two files with ``oracle/ref_host.cpp`` into a host library that
  runs the reference's smoothing, mute, stability check and padding on the
  CPU (``smooth_model``, ``mute``, ``stability``, ``expand_model``).

Only the tests and the bench's baselines use this, as checkers and as the
reference's timings next to the engine's.  The reference's update kernels
damp U(t) in place while neighbouring threads read it (cpp/Modeling.cu:535-550),
so their output inside the absorbing border depends on the order in which
thread blocks run.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from .oracle import APPROX, Grid, Models

_LIB = None


def cubin_path():
    """Path of the reference cubin, or None when it was not built here."""
    p = _build.build_ref_cubin()
    return p if p and os.path.exists(p) else None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build_harness()
        if path is None:
            raise RuntimeError("CUDA headers not found: cannot build the reference-kernel harness")
        L = ctypes.CDLL(path)
        p, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_forward.restype = i
        L.ref_forward.argtypes = [ctypes.c_char_p, i, i, i, i, f, f, f, i, i, p, p, p, p, p, p, i, p, p, i, p, p, p,
                                  ctypes.POINTER(ctypes.c_double)]
        L.ref_rtm.restype = i
        L.ref_rtm.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i, i, i, i, f, f, f, i, i, p, p, p, p, p, p, i, p, p,
                              i, p, p, p, i, p, p, ctypes.POINTER(ctypes.c_double)]
        L.ref_last_error.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def migration_cubin_path():
    """Path of the cubin of the reference's migration kernels (cpp/Migration.cu),
    or None when it was not built here."""
    p = _build.build_ref_migration_cubin()
    return p if p and os.path.exists(p) else None


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def forward(g: Grid, m: Models, wavelet, sx, sz, rx, rz):
    """Seismograms [nshots][nt_data][nrec] of the reference kernels (Cerjan
    boundaries: the reference C++ has no CPML) and their device time in ms.
    sx, sz, rx, rz are expanded-grid indices."""
    if g.abc != "cerjan":
        raise ValueError("the reference's CUDA kernels implement Cerjan boundaries only")
    cubin = cubin_path()
    if cubin is None:
        raise RuntimeError("the reference cubin is not available")
    c = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    vp, eps, dl, th = c(m.vp), c(m.eps), c(m.delta), c(m.theta)
    A = c(m.A)
    w = c(wavelet)
    sx, sz = np.ascontiguousarray(sx, np.int32), np.ascontiguousarray(sz, np.int32)
    rx, rz = np.ascontiguousarray(rx, np.int32), np.ascontiguousarray(rz, np.int32)
    seis = np.zeros((sx.size, g.nt_data, rx.size), np.float32)
    ms = ctypes.c_double(0.0)
    rc = lib().ref_forward(cubin.encode(), APPROX[g.approx], g.nz_a, g.nx_a, g.N, g.dz, g.dx, g.dt, g.nt, g.itlag,
                           _ptr(vp), _ptr(eps), _ptr(dl), _ptr(th), _ptr(A), _ptr(w), sx.size, _ptr(sz), _ptr(sx),
                           rx.size, _ptr(rz), _ptr(rx), _ptr(seis), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().ref_last_error().decode())
    return seis, ms.value


def rtm(g: Grid, m: Models, wavelet, sx, sz, rx, rz, obs, normalize=True):
    """Image and illumination [nz][nx] of the reference's on-the-fly migration
    (cpp/Migration.cu:359-397) run with its own forward and migration kernels
    (Cerjan boundaries), summed over the shots, and the device time in ms.
    obs [nshots][nt_data][nrec] is the observed data; sx, sz, rx, rz are
    expanded-grid indices; normalize applies the C++ normalizeImage."""
    if g.abc != "cerjan":
        raise ValueError("the reference's CUDA kernels implement Cerjan boundaries only")
    cm, cg = cubin_path(), migration_cubin_path()
    if cm is None or cg is None:
        raise RuntimeError("the reference cubins are not available")
    c = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    vp, eps, dl, th = c(m.vp), c(m.eps), c(m.delta), c(m.theta)
    sx, sz = np.ascontiguousarray(sx, np.int32), np.ascontiguousarray(sz, np.int32)
    rx, rz = np.ascontiguousarray(rx, np.int32), np.ascontiguousarray(rz, np.int32)
    d = np.ascontiguousarray(obs, np.float32)
    assert d.shape == (sx.size, g.nt_data, rx.size)
    nzi, nxi = g.nz_a - 2 * g.N, g.nx_a - 2 * g.N
    img = np.zeros((nzi, nxi), np.float32)
    ilum = np.zeros((nzi, nxi), np.float32)
    ms = ctypes.c_double(0.0)
    rc = lib().ref_rtm(cm.encode(), cg.encode(), APPROX[g.approx], g.nz_a, g.nx_a, g.N, g.dz, g.dx, g.dt, g.nt,
                       g.itlag, _ptr(vp), _ptr(eps), _ptr(dl), _ptr(th), _ptr(c(m.A)), _ptr(c(wavelet)), sx.size,
                       _ptr(sz), _ptr(sx), rx.size, _ptr(rz), _ptr(rx), _ptr(d), 1 if normalize else 0, _ptr(img),
                       _ptr(ilum), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().ref_last_error().decode())
    return img, ilum, ms.value


_HOST = None


def host_lib():
    """The reference's own host routines (cpp/Migration.cu, cpp/Modeling.cu
    through oracle/ref_host.cpp), or None when the reference sources were
    absent where this checkout was built."""
    global _HOST
    if _HOST is None:
        path = _build.build_ref_host()
        if path is None or not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        p, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_smooth_model.restype = i
        L.ref_smooth_model.argtypes = [p, i, i, f, i, p]
        L.ref_mute.restype = i
        L.ref_mute.argtypes = [p, i, i, p, p, f, f, f, f, f, f]
        L.ref_stability.restype = i
        L.ref_stability.argtypes = [i, i, i, p, p, p, p, f, f, f, f, ctypes.c_char_p, i]
        L.ref_expand_model.restype = i
        L.ref_expand_model.argtypes = [p, i, i, i, p]
        _HOST = L
    return _HOST


def _need():
    L = host_lib()
    if L is None:
        raise RuntimeError("the reference's host routines were not built (reference sources absent)")
    return L


def smooth_model(f, sigma, parameter=False, water_model=None):
    """Migration::createMask(water_model) then Migration::smoothModel(f, mask,
    parameter), both the reference's compiled code; returns a new array."""
    L = _need()
    out = np.ascontiguousarray(f, dtype=np.float32).copy()
    w = np.ascontiguousarray(f if water_model is None else water_model, dtype=np.float32).copy()
    assert w.shape == out.shape
    L.ref_smooth_model(_ptr(out), out.shape[0], out.shape[1], float(sigma), 1 if parameter else 0, _ptr(w))
    return out


def mute(seis, rec_x, rec_z, shot_x, shot_z, dt, v0, shift, window):
    """Migration::Mute of one shot's gather [nt][nrec] (compiled reference
    code); returns a new array."""
    L = _need()
    out = np.ascontiguousarray(seis, dtype=np.float32).copy()
    rx = np.ascontiguousarray(rec_x, dtype=np.float32)
    rz = np.ascontiguousarray(rec_z, dtype=np.float32)
    L.ref_mute(_ptr(out), out.shape[0], out.shape[1], _ptr(rx), _ptr(rz), float(shot_x), float(shot_z), float(dt),
               float(v0), float(shift), float(window))
    return out


def expand_model(model, N):
    """Modeling::expandModel (compiled reference code): edge-replicating
    padding by N cells; returns [nz + 2N][nx + 2N]."""
    L = _need()
    m = np.ascontiguousarray(model, dtype=np.float32)
    out = np.zeros((m.shape[0] + 2 * N, m.shape[1] + 2 * N), np.float32)
    L.ref_expand_model(_ptr(m), m.shape[0], m.shape[1], int(N), _ptr(out))
    return out


def stability(approx, vp, eps=None, delta=None, theta_deg=None, dx=10.0, dz=10.0, dt=1e-3, fcut=30.0):
    """Modeling::checkDispersionAndStability (compiled reference code) on
    unpadded [nz][nx] models; returns its report parsed into a dict of floats
    (printed with 9 significant digits, so every value is exact) and the two
    verdict flags."""
    L = _need()
    a = {"acoustic": 0, "VTI": 1, "TTI": 2}[approx]
    arrs = [None if v is None else np.ascontiguousarray(v, dtype=np.float32) for v in (vp, eps, delta, theta_deg)]
    buf = ctypes.create_string_buffer(8192)
    nz, nx = arrs[0].shape
    rc = L.ref_stability(a, nz, nx, *[_ptr(v) for v in arrs], float(dx), float(dz), float(dt), float(fcut), buf,
                         len(buf))
    assert rc == 0
    text = buf.value.decode()
    keys = {"Minimum velocity": "vp_min", "Maximum velocity": "vp_max", "Critical dx for dispersion": "dx_lim",
            "Critical dz for dispersion": "dz_lim", "Critical dt for stability": "dt_lim",
            "Maximum epsilon": "eps_max", "Maximum delta": "delta_max"}
    out = {"satisfied": "conditions satisfied" in text, "text": text}
    for line in text.splitlines():
        for k, name in keys.items():
            if line.startswith(f"info: {k}:"):
                out[name] = np.float32(float(line.rsplit(":", 1)[1].split()[0]))
    return out
