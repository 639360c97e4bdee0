"""CPU oracle: restatement of the reference hot path, for checking only.

TEST INFRASTRUCTURE.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg import this module; the product path never does.

Host-side pieces are restated here in numpy; the stencil steps run in the C
restatement ``pam_oracle.c`` (FP32 with the reference's term order, or FP64).
Every function cites the reference code it follows.
"""
import ctypes
import math
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import build as _build

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        for sfx, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            p = ctypes.c_void_p
            i = ctypes.c_int
            getattr(L, "og_step_" + sfx).argtypes = [i, i, i, i, ct, ct, ct] + [p] * 15
            getattr(L, "og_adjoint_products_" + sfx).argtypes = [i, i, i, ct, ct] + [p] * 10
            getattr(L, "og_rtm_step_" + sfx).argtypes = [i, i, i, i, ct, ct, ct] + [p] * 19
            getattr(L, "og_adjoint_exact_step_" + sfx).argtypes = [i, i, i, ct, ct, ct] + [p] * 5
        L.og_threads.restype = ctypes.c_int
        L.og_set_threads.argtypes = [ctypes.c_int]
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


APPROX = {"acoustic": 0, "VTI": 1, "TTI": 2}


@dataclass
class Grid:
    """Geometry of one modelling job on the expanded grid (cpp/Survey.hpp:20-48)."""
    nz: int              # interior rows
    nx: int              # interior columns
    N: int               # absorbing width N_abc
    dz: float
    dx: float
    dt: float
    nt: int              # itlag + nt_data
    itlag: int
    fcut: float
    approx: str = "acoustic"
    abc: str = "cerjan"

    @property
    def nz_a(self):
        return self.nz + 2 * self.N

    @property
    def nx_a(self):
        return self.nx + 2 * self.N

    @property
    def nt_data(self):
        return self.nt - self.itlag


# ---------------------------------------------------------------- host-side restatements

def ricker_cpp(nt, dt, fcut, tlag, dx, dz):
    """Ricker wavelet of cpp/Modeling.cu:84-100, float32 arithmetic."""
    f = np.float32
    pi = f(3.14159265358979323846)
    fc = f(fcut) / (f(3.0) * np.sqrt(pi, dtype=f))
    scale = f(1.0) / (f(dx) * f(dz))
    n = np.arange(nt, dtype=f)
    td = n * f(dt) - f(tlag)
    arg = pi * pi * pi * fc * fc * td * td
    return ((f(1.0) - f(2.0) * arg) * np.exp(-arg, dtype=f) * scale).astype(f)


def cerjan_vector(N):
    """Cerjan factors of cpp/Modeling.cu:111-120, float32 arithmetic."""
    f = np.float32
    sb = f(3.0) * f(N)
    i = np.arange(N, dtype=f)
    fb = (f(N) - i) / (f(1.4142) * sb)
    return np.exp(-fb * fb, dtype=f).astype(f)


def expand_model(m, N):
    """Edge-replicating padding of cpp/Modeling.cu:130-182."""
    return np.pad(np.asarray(m), N, mode="edge")


def cpml_profiles(vp_exp, N, dx, dz, dt, fcut):
    """CPML a/b coefficients of src/utils.py:198-240 with the constants of
    src/Modeling2D.py:110-126, in float64.  Returns full-grid (ax, bx, az, bz);
    entries outside the strips are (1, 0)."""
    R = 1e-3 ** (N / 10) if N < 200 else 1e-3 ** (150 / 10)
    d0 = -(2 + 1) * math.log(R)
    f_pico = fcut / 3
    nz, nx = vp_exp.shape
    vp = vp_exp.astype(np.float64)

    def prof(n, h, idx):
        pts = np.zeros(n)
        inside = np.zeros(n, dtype=bool)
        lo = idx < N
        hi = idx >= n - N
        pts[lo] = (N - idx[lo] - 1.0) * h
        pts[hi] = (idx[hi] - n + N) * h
        inside[lo | hi] = True
        r = pts / (N * h)
        return r, inside

    rx, inx = prof(nx, dx, np.arange(nx))
    rz, inz = prof(nz, dz, np.arange(nz))
    dX = np.where(inx[None, :], d0 / (2 * N * dx) * rx[None, :] ** 2 * vp, 0.0)
    alX = np.where(inx[None, :], np.pi * f_pico * (1.0 - rx[None, :] ** 2), 0.0) * np.ones((nz, 1))
    dZ = np.where(inz[:, None], d0 / (2 * N * dz) * rz[:, None] ** 2 * vp, 0.0)
    alZ = np.where(inz[:, None], np.pi * f_pico * (1.0 - rz[:, None] ** 2), 0.0) * np.ones((1, nx))
    ax = np.exp(-(dX + alX) * dt)
    az = np.exp(-(dZ + alZ) * dt)
    with np.errstate(invalid="ignore", divide="ignore"):
        bx = np.where(np.abs(dX + alX) > 1e-10, dX / (dX + alX) * (ax - 1.0), 0.0)
        bz = np.where(np.abs(dZ + alZ) > 1e-10, dZ / (dZ + alZ) * (az - 1.0), 0.0)
    return ax, bx, az, bz


def mute(seis, rec_x, rec_z, sx, sz, dt, shift, window, v0):
    """Top mute of cpp/Migration.cu:86-115 (float32)."""
    f = np.float32
    s = np.array(seis, dtype=f, copy=True)
    nt = s.shape[0]
    for r in range(s.shape[1]):
        ddz = f(rec_z[r]) - f(sz)
        ddx = f(rec_x[r]) - f(sx)
        dist = np.sqrt(ddz * ddz + ddx * ddx, dtype=f)
        t1 = dist / f(v0) + f(shift)
        t2 = t1 + f(window)
        for it in range(nt):
            t = f(it) * f(dt)
            if t < t1:
                s[it, r] = 0.0
            elif t < t2:
                s[it, r] = s[it, r] * ((t - t1) / (t2 - t1))
    return s


def gaussian_taps_cpp(sigma):
    """Migration::gaussianFilter1D (cpp/Migration.cu:145-169): length
    ceil(6 sigma + 1) made odd, taps exp(-(x*x) / (2 sigma sigma)) in float
    (the C library's expf, which the exponential in double rounded to float
    reproduces for these arguments; numpy's float32 exp does not), divided by
    their sum accumulated in order."""
    sg = np.float32(sigma)
    ks = int(math.ceil(np.float32(6.0) * sg + np.float32(1.0)))
    if ks % 2 == 0:
        ks += 1
    half = ks // 2
    den = np.float32(np.float32(2.0) * sg) * sg
    k = np.empty(ks, np.float32)
    total = np.float32(0.0)
    for i in range(ks):
        x = i - half
        k[i] = np.float32(math.exp(float(np.float32(-(x * x)) / den)))
        total = np.float32(total + k[i])
    return (k / total).astype(np.float32)


def water_mask_cpp(model):
    """Migration::createMask (cpp/Migration.cu:131-143): cells within 1e-3 of
    the model's minimum."""
    m = np.asarray(model, dtype=np.float32)
    return np.abs(m - m.min()) < np.float32(1e-3)


def smooth_model_cpp(f_in, sigma, parameter=False, water_model=None):
    """Migration::smoothModel (cpp/Migration.cu:171-236): separable Gaussian
    smoothing of the slowness 1/f (velocity, parameter False) or of the value
    (parameter True), indices clamped at the edges, the x pass then the z pass,
    each tap sum accumulated in float from the first tap to the last; cells of
    the water mask keep their value.  The reference derives the mask from the
    unsmoothed velocity for every field it smooths (cpp/Migration.cu:265-290):
    water_model is that velocity (None: f_in itself)."""
    f = np.asarray(f_in, dtype=np.float32)
    mask = water_mask_cpp(f if water_model is None else water_model)
    k = gaussian_taps_cpp(sigma)
    half = k.size // 2
    s_old = f.copy() if parameter else (np.float32(1.0) / f).astype(np.float32)
    nz, nx = f.shape
    tmp = np.zeros_like(s_old)
    for i in range(k.size):
        xi = np.clip(np.arange(nx) + i - half, 0, nx - 1)
        tmp = (tmp + (k[i] * s_old[:, xi]).astype(np.float32)).astype(np.float32)
    s = np.zeros_like(s_old)
    for i in range(k.size):
        zi = np.clip(np.arange(nz) + i - half, 0, nz - 1)
        s = (s + (k[i] * tmp[zi, :]).astype(np.float32)).astype(np.float32)
    s = np.where(mask, s_old, s)
    return s if parameter else (np.float32(1.0) / s).astype(np.float32)


def laplacian_filter(img, dz, dx):
    """Image Laplacian post-filter of src/Viewdata.py:23-41 (2nd order,
    edges copied, sign flipped)."""
    f = np.asarray(img, dtype=np.float64)
    g = np.zeros_like(f)
    g[1:-1, 1:-1] = ((f[2:, 1:-1] + f[:-2, 1:-1] - 2 * f[1:-1, 1:-1]) / (dz * dz)
                     + (f[1:-1, 2:] + f[1:-1, :-2] - 2 * f[1:-1, 1:-1]) / (dx * dx))
    g[0, :] = g[1, :]
    g[-1, :] = g[-2, :]
    g[:, 0] = g[:, 1]
    g[:, -1] = g[:, -2]
    return -g


# ---------------------------------------------------------------- stepping

@dataclass
class Models:
    """Expanded-grid model arrays (theta in radians)."""
    vp: np.ndarray
    eps: Optional[np.ndarray] = None
    delta: Optional[np.ndarray] = None
    theta: Optional[np.ndarray] = None
    cpml: Optional[tuple] = None          # (ax, bx, az, bz) float64 full grid
    A: Optional[np.ndarray] = None        # Cerjan vector

    @staticmethod
    def build(g: Grid, vp, eps=None, delta=None, theta_deg=None):
        """Expand interior models and precompute the boundary tables, like
        Modeling::setModel (cpp/Modeling.cu:329-382)."""
        vpe = expand_model(np.asarray(vp, np.float32), g.N).astype(np.float32)
        m = Models(vp=vpe)
        if g.approx in ("VTI", "TTI"):
            m.eps = expand_model(np.asarray(eps, np.float32), g.N).astype(np.float32)
            m.delta = expand_model(np.asarray(delta, np.float32), g.N).astype(np.float32)
        if g.approx == "TTI":
            th = (np.asarray(theta_deg, np.float32) * np.float32(3.14159265358979323846)
                  / np.float32(180.0)).astype(np.float32)
            m.theta = expand_model(th, g.N).astype(np.float32)
        if g.abc == "CPML":
            m.cpml = cpml_profiles(vpe, g.N, g.dx, g.dz, g.dt, g.fcut)
        else:
            m.A = cerjan_vector(g.N)
        return m


class _State:
    def __init__(self, g: Grid, m: Models, dtype):
        self.g, self.m, self.dt = g, m, dtype
        shp = (g.nz_a, g.nx_a)
        self.cur = np.zeros(shp, dtype)
        self.fut = np.zeros(shp, dtype)
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype)
        self.vp, self.eps, self.delta, self.theta = c(m.vp), c(m.eps), c(m.delta), c(m.theta)
        self.A = c(m.A)
        if m.cpml is not None:
            self.ab = [c(a) for a in m.cpml]
            self.mem = [np.zeros(shp, dtype) for _ in range(4)]
        else:
            self.ab = [None] * 4
            self.mem = [None] * 4

    def step(self, cur=None, fut=None, mem=None):
        g = self.g
        cur = self.cur if cur is None else cur
        fut = self.fut if fut is None else fut
        mem = self.mem if mem is None else mem
        f = lib().og_step_f32 if self.dt == np.float32 else lib().og_step_f64
        f(APPROX[g.approx], g.nz_a, g.nx_a, g.N, g.dz, g.dx, g.dt,
          _p(fut), _p(cur), _p(self.vp), _p(self.eps), _p(self.delta), _p(self.theta),
          _p(self.A), *[_p(a) for a in mem], *[_p(a) for a in self.ab])


def step(g: Grid, m: Models, Uf, Uc, mem=None, dtype=np.float64):
    """One forward step on caller arrays (kernel-level checks)."""
    st = _State(g, m, dtype)
    st.step(cur=Uc, fut=Uf, mem=mem if mem is not None else st.mem)


def forward_shot(g: Grid, m: Models, src, sx, sz, rx, rz, dtype=np.float64, save=False,
                 on_step=None):
    """Shot loop of Modeling::solveWaveEquation (cpp/Modeling.cu:433-479):
    inject, step, record U(t) after the step for t >= itlag, swap.
    Returns the seismogram [nt_data][Nrec] (and every post-step U(t) if save)."""
    st = _State(g, m, dtype)
    seis = np.zeros((g.nt_data, len(rx)), dtype)
    rx = np.asarray(rx)
    rz = np.asarray(rz)
    saved = [] if save else None
    for k in range(g.nt):
        st.cur[sz, sx] += dtype(src[k])
        st.step()
        if k >= g.itlag:
            seis[k - g.itlag] = st.cur[rz, rx]
        if save:
            saved.append(st.cur.copy())
        if on_step is not None:
            on_step(k, st)
        st.cur, st.fut = st.fut, st.cur
    return (seis, saved) if save else seis


def rtm_shot(g: Grid, m: Models, src, sx, sz, rx, rz, dobs, dtype=np.float64):
    """On-the-fly RTM of one shot, Migration::solveReverseTimeMigrationOntheFly
    (cpp/Migration.cu:359-397): store the source field every step, then run
    the receiver field back from t = nt-1 to 0, injecting d(t)/(dx dz)
    (cpp/Migration.cu:493-502) and applying the imaging condition.
    Returns (image, ilum) on the interior [nz][nx], not normalised."""
    _, P = forward_shot(g, m, src, sx, sz, rx, rz, dtype=dtype, save=True)
    st = _State(g, m, dtype)
    img = np.zeros((g.nz, g.nx), dtype)
    ilum = np.zeros((g.nz, g.nx), dtype)
    shp = (g.nz_a, g.nx_a)
    prods = [np.zeros(shp, dtype) for _ in range(5)]
    L = lib()
    rstep = L.og_rtm_step_f32 if dtype == np.float32 else L.og_rtm_step_f64
    prod = L.og_adjoint_products_f32 if dtype == np.float32 else L.og_adjoint_products_f64
    inv = dtype(1.0) / (dtype(g.dx) * dtype(g.dz))
    rx = np.asarray(rx)
    rz = np.asarray(rz)
    a = APPROX[g.approx]
    for t in range(g.nt - 1, -1, -1):
        if t >= g.itlag:
            np.add.at(st.cur, (rz, rx), np.asarray(dobs[t - g.itlag], dtype) * inv)
        if a != 0:
            prod(a, g.nz_a, g.nx_a, g.dz, g.dx, _p(st.cur), _p(P[t]), _p(st.eps), _p(st.delta),
                 _p(st.theta), _p(prods[0]), _p(prods[1]), _p(prods[2] if a == 2 else None),
                 _p(prods[3]), _p(prods[4]))
        rstep(a, g.nz_a, g.nx_a, g.N, g.dz, g.dx, g.dt, _p(st.fut), _p(st.cur), _p(P[t]),
              _p(img), _p(ilum), _p(st.vp), *[_p(x) for x in prods], _p(st.A),
              *[_p(x) for x in st.mem], *[_p(x) for x in st.ab])
        st.cur, st.fut = st.fut, st.cur
    return img, ilum


def normalize_image_cpp(img, ilum):
    """cpp/Migration.cu:470-484: img/ilum where ilum > 1e-12, else 0."""
    img = np.asarray(img, np.float64)
    ilum = np.asarray(ilum, np.float64)
    out = np.zeros_like(img)
    m = ilum > 1e-12
    out[m] = img[m] / ilum[m]
    return out


def fwi_gradient_shot(g: Grid, m: Models, src, sx, sz, rx, rz, resid, dtype=np.float64):
    """FWI gradient of one shot in the reference form.

    Per-cell formula of cpp/inversion.cu:142-213 (updateAdjointWaveEquationandGradient):
    the receiver field is the forward operator driven by resid/(dx dz), and
    g += Ub(t) * (P(t+1) - 2 P(t) + P(t-1)) / dt^2 on the interior.  The
    C++ driver for that kernel does not compile, so the loop follows
    src/Migration.py:1030-1049: t = nt-2 .. 1, illumination sum of P(t)^2 over
    all forward steps.  Returns (grad, ilum), un-normalised."""
    _, P = forward_shot(g, m, src, sx, sz, rx, rz, dtype=dtype, save=True)
    st = _State(g, m, dtype)
    grad = np.zeros((g.nz, g.nx), dtype)
    ilum = np.zeros((g.nz, g.nx), dtype)
    N = g.N
    sl = (slice(N, N + g.nz), slice(N, N + g.nx))
    for k in range(g.nt):
        ilum += P[k][sl] * P[k][sl]
    inv = dtype(1.0) / (dtype(g.dx) * dtype(g.dz))
    idt2 = dtype(1.0) / (dtype(g.dt) * dtype(g.dt))
    rx = np.asarray(rx)
    rz = np.asarray(rz)
    for t in range(g.nt - 2, 0, -1):
        if t >= g.itlag:
            np.add.at(st.cur, (rz, rx), np.asarray(resid[t - g.itlag], dtype) * inv)
        adj = st.cur[sl].copy()
        grad += adj * ((P[t + 1][sl] - dtype(2.0) * P[t][sl] + P[t - 1][sl]) * idt2)
        st.step()
        st.cur, st.fut = st.fut, st.cur
    return grad, ilum


_C8 = (-1435.0 / 504.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0)
_A8 = (4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0)


def multiparameter_gradient_terms(cur, adj, eps, delta, theta, dx, dz):
    """Per-cell multiparameter gradient increments of src/utils.py:1309-1463
    (calculateGradientVTI / calculateGradientTTI), in float64 like the
    reference's numba code, on [4, nz-4) x [4, nx-4) of the interior arrays
    passed (zero elsewhere).  theta is in radians, None for VTI.
    Returns (d_eps, d_delta, d_theta or None)."""
    U = np.asarray(cur, np.float64)
    A = np.asarray(adj, np.float64)
    nz, nx = U.shape
    c = slice(4, nz - 4), slice(4, nx - 4)

    def sh(dzi, dxi):
        return U[4 + dzi:nz - 4 + dzi, 4 + dxi:nx - 4 + dxi]

    pxx = (_C8[0] * sh(0, 0) + sum(_C8[k] * (sh(0, k) + sh(0, -k)) for k in range(1, 5))) / (dx * dx)
    pzz = (_C8[0] * sh(0, 0) + sum(_C8[k] * (sh(k, 0) + sh(-k, 0)) for k in range(1, 5))) / (dz * dz)
    px = sum(_A8[k - 1] * (sh(0, k) - sh(0, -k)) for k in range(1, 5)) / dx
    pz = sum(_A8[k - 1] * (sh(k, 0) - sh(-k, 0)) for k in range(1, 5)) / dz
    e = np.asarray(eps, np.float64)[c]
    d = np.asarray(delta, np.float64)[c]
    out_e, out_d = np.zeros_like(U), np.zeros_like(U)
    out_t = None
    with np.errstate(divide="ignore", invalid="ignore"):
        if theta is None:
            h, q = px, pz
        else:
            th = np.asarray(theta, np.float64)[c]
            pxz = sum(_A8[m - 1] * _A8[n - 1] * (sh(n, m) - sh(-n, m) + sh(-n, -m) - sh(n, -m))
                      for m in range(1, 5) for n in range(1, 5)) / (dz * dx)
            h = px * np.cos(th) - pz * np.sin(th)
            q = px * np.sin(th) + pz * np.cos(th)
        num = -2.0 * (e - d) * (h * h) * (q * q)
        den = (1.0 + 2.0 * e) * h ** 4 + q ** 4 + 2.0 * (1.0 + d) * (h * h) * (q * q)
        ok = np.abs(den) >= 1e-150
        den2 = np.where(ok, den * den, 1.0)
        dSd_de = np.where(ok, (-2.0 * h * h * q * q * den - num * 2.0 * h ** 4) / den2, 0.0)
        dSd_dd = np.where(ok, (2.0 * h * h * q * q * den - num * 2.0 * h * h * q * q) / den2, 0.0)
        if theta is None:
            out_e[c] = A[c] * ((-2.0 - dSd_de) * pxx - dSd_de * pzz)
            out_d[c] = A[c] * (-dSd_dd * (pxx + pzz))
        else:
            dnum_dt = -2.0 * (e - d) * (-2.0 * h * q ** 3 + 2.0 * h ** 3 * q)
            dden_dt = (-4.0 * (1.0 + 2.0 * e) * h ** 3 * q + 4.0 * h * q ** 3
                       + 2.0 * (1.0 + d) * (-2.0 * h * q ** 3 + 2.0 * h ** 3 * q))
            dSd_dt = np.where(ok, (dnum_dt * den - num * dden_dt) / den2, 0.0)
            s2 = np.sin(2.0 * th)
            dA = 2.0 * e * s2 - dSd_dt
            dB = -2.0 * e * s2 - dSd_dt
            dC = 4.0 * e * np.cos(2.0 * th)
            out_e[c] = A[c] * (-(2.0 * np.cos(th) ** 2 + dSd_de) * pxx - (2.0 * np.sin(th) ** 2 + dSd_de) * pzz
                               + 2.0 * s2 * pxz)
            out_d[c] = A[c] * (-dSd_dd * (pxx + pzz))
            out_t = np.zeros_like(U)
            out_t[c] = A[c] * (dA * pxx + dB * pzz + dC * pxz)
    return out_e, out_d, out_t


def multiparameter_fwi_gradient_shot(g: Grid, m: Models, src, sx, sz, rx, rz, resid, dtype=np.float64):
    """The reference FWI gradient of one VTI/TTI shot with the multiparameter
    terms (the backward loops of src/Migration.py with fwi and multiparameter
    set): receiver field of the reference's anisotropic adjoint
    (cpp/Migration.cu:573-973) driven by resid/(dx dz), for t = nt-2 .. 1
    g_vp += adj (P(t+1) - 2P(t) + P(t-1))/dt^2 and the per-cell epsilon, delta
    (theta) terms of multiparameter_gradient_terms on the interior; the
    illumination sums P(t)^2 over all steps.
    Returns (g_vp, g_eps, g_delta, g_theta or None, ilum), un-normalised."""
    _, P = forward_shot(g, m, src, sx, sz, rx, rz, dtype=dtype, save=True)
    st = _State(g, m, dtype)
    N = g.N
    sl = (slice(N, N + g.nz), slice(N, N + g.nx))
    ilum = np.zeros((g.nz, g.nx), np.float64)
    for k in range(g.nt):
        ilum += np.asarray(P[k][sl], np.float64) ** 2
    gvp = np.zeros((g.nz, g.nx), np.float64)
    ge = np.zeros((g.nz, g.nx), np.float64)
    gd = np.zeros((g.nz, g.nx), np.float64)
    gt = np.zeros((g.nz, g.nx), np.float64) if g.approx == "TTI" else None
    shp = (g.nz_a, g.nx_a)
    prods = [np.zeros(shp, dtype) for _ in range(5)]
    dummy_img = np.zeros((g.nz, g.nx), dtype)
    dummy_ilum = np.zeros((g.nz, g.nx), dtype)
    L = lib()
    rstep = L.og_rtm_step_f32 if dtype == np.float32 else L.og_rtm_step_f64
    prod = L.og_adjoint_products_f32 if dtype == np.float32 else L.og_adjoint_products_f64
    inv = dtype(1.0) / (dtype(g.dx) * dtype(g.dz))
    idt2 = 1.0 / (float(g.dt) * float(g.dt))
    rx = np.asarray(rx)
    rz = np.asarray(rz)
    a = APPROX[g.approx]
    eps_i = np.asarray(m.eps, np.float64)[sl]
    del_i = np.asarray(m.delta, np.float64)[sl]
    th_i = None if m.theta is None else np.asarray(m.theta, np.float64)[sl]
    for t in range(g.nt - 2, 0, -1):
        if t >= g.itlag:
            np.add.at(st.cur, (rz, rx), np.asarray(resid[t - g.itlag], dtype) * inv)
        adj = np.asarray(st.cur[sl], np.float64)
        gvp += adj * ((np.asarray(P[t + 1][sl], np.float64) - 2.0 * np.asarray(P[t][sl], np.float64)
                       + np.asarray(P[t - 1][sl], np.float64)) * idt2)
        de, dd, dth = multiparameter_gradient_terms(P[t][sl], adj, eps_i, del_i, th_i, g.dx, g.dz)
        ge += de
        gd += dd
        if gt is not None:
            gt += dth
        prod(a, g.nz_a, g.nx_a, g.dz, g.dx, _p(st.cur), _p(P[t]), _p(st.eps), _p(st.delta),
             _p(st.theta), _p(prods[0]), _p(prods[1]), _p(prods[2] if a == 2 else None),
             _p(prods[3]), _p(prods[4]))
        rstep(a, g.nz_a, g.nx_a, g.N, g.dz, g.dx, g.dt, _p(st.fut), _p(st.cur), _p(P[t]),
              _p(dummy_img), _p(dummy_ilum), _p(st.vp), *[_p(x) for x in prods], _p(st.A),
              *[_p(x) for x in st.mem], *[_p(x) for x in st.ab])
        st.cur, st.fut = st.fut, st.cur
    return gvp, ge, gd, gt, ilum


def misfit_and_exact_gradient(g: Grid, m: Models, src, sx, sz, rx, rz, dobs, dtype=np.float64):
    """L2 misfit J = 1/2 sum (d - dobs)^2 and its exact discrete gradient with
    respect to the expanded-grid kappa = vp^2 dt^2, for the acoustic Cerjan
    scheme (transpose of forward_shot; no reference counterpart).  Returns
    (J, dJ/dkappa on the expanded grid)."""
    assert g.approx == "acoustic" and g.abc == "cerjan"
    d, C = forward_shot(g, m, src, sx, sz, rx, rz, dtype=dtype, save=False), None
    # keep the injected pre-step fields c~(t) (cpp/Modeling.cu:447) and D c~(t)
    ctil = []
    st = _State(g, m, dtype)
    rxa, rza = np.asarray(rx), np.asarray(rz)
    for k in range(g.nt):
        st.cur[sz, sx] += dtype(src[k])
        ctil.append(st.cur.copy())
        st.step()
        st.cur, st.fut = st.fut, st.cur
    r = (d - np.asarray(dobs, dtype))
    J = 0.5 * float(np.sum(r.astype(np.float64) ** 2))
    nz, nx, N = g.nz_a, g.nx_a, g.N
    Dm = np.ones((nz, nx), dtype)
    A = st.A
    for x in range(nx):
        if x < N:
            Dm[:, x] *= A[x]
        if x >= nx - N:
            Dm[:, x] *= A[nx - 1 - x]
    for z in range(nz):
        if z < N:
            Dm[z, :] *= A[z]
        if z >= nz - N:
            Dm[z, :] *= A[nz - 1 - z]
    Dm[:4, :] = Dm[-4:, :] = 1
    Dm[:, :4] = Dm[:, -4:] = 1
    lam_next = np.zeros((nz, nx), dtype)      # l(t+1)
    lam_next2 = np.zeros((nz, nx), dtype)     # l(t+2)
    work = np.zeros((nz, nx), dtype)
    gk = np.zeros((nz, nx), dtype)
    upd = np.zeros((nz, nx), bool)
    upd[4:-4, 4:-4] = True
    L = lib()
    astep = L.og_adjoint_exact_step_f32 if dtype == np.float32 else L.og_adjoint_exact_step_f64
    vp = st.vp
    kap = vp.astype(dtype) * vp.astype(dtype) * dtype(g.dt) * dtype(g.dt)
    for t in range(g.nt - 1, -1, -1):
        # l(t) = 2 D l(t+1) + L(k D l(t+1)) - D^2 l(t+2) + D R^T r(t)
        buf = lam_next2.copy()
        astep(nz, nx, N, g.dz, g.dx, g.dt, _p(buf), _p(lam_next), _p(vp), _p(A), _p(work))
        lam_t = np.where(upd, buf, 0).astype(dtype)
        if t >= g.itlag:
            np.add.at(lam_t, (rza, rxa), r[t - g.itlag] * Dm[rza, rxa])
        # gradient: c(t+1) = D(2c~ + k L c~ - D c~(t-1)) -> dJ/dk += l(t+1) D L c~(t)
        if t < g.nt - 1:
            c = ctil[t]
            lap = np.zeros((nz, nx), dtype)
            lap[4:-4, 4:-4] = _lap(c, g.dz, g.dx, dtype)
            gk += lam_next * Dm * lap
        lam_next2, lam_next = lam_next, lam_t
    return J, gk


def _lap(U, dz, dx, dtype):
    c = [-1435.0 / 504.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0]
    nz, nx = U.shape
    U = U.astype(np.float64)
    out = c[0] * U[4:-4, 4:-4] * (1.0 / (dx * dx) + 1.0 / (dz * dz))
    for k in range(1, 5):
        out = out + c[k] * (U[4:-4, 4 + k:nx - 4 + k] + U[4:-4, 4 - k:nx - 4 - k]) / (dx * dx)
        out = out + c[k] * (U[4 + k:nz - 4 + k, 4:-4] + U[4 - k:nz - 4 - k, 4:-4]) / (dz * dz)
    return out.astype(dtype)
