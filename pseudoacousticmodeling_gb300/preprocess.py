"""Host-side preparation steps of the reference, vectorised with numpy.

Each runs once per job or per shot, off the GPU time line:
  ricker / ricker_half_derivative  source wavelets (cpp/Modeling.cu:84-100,
                                   src/utils.py:21-28)
  mute                             top mute of observed data (cpp/Migration.cu:86-115)
  smooth_model                     separable Gaussian smoothing with the water
                                   layer kept (cpp/Migration.cu:131-236)
  laplacian_filter                 image post-filter (src/Viewdata.py:23-41)
"""
import math

import numpy as np

F32 = np.float32
PI32 = F32(3.14159265358979323846)


def ricker(nt, dt, fcut, dx, dz):
    """Ricker wavelet scaled by 1/(dx dz), float32 arithmetic as in the C++
    modeller; delayed by tlag = 2 sqrt(pi)/fcut."""
    tlag = F32(2.0) * np.sqrt(PI32, dtype=F32) / F32(fcut)
    fc = F32(fcut) / (F32(3.0) * np.sqrt(PI32, dtype=F32))
    td = np.arange(nt, dtype=F32) * F32(dt) - tlag
    arg = PI32 * PI32 * PI32 * fc * fc * td * td
    return ((F32(1.0) - F32(2.0) * arg) * np.exp(-arg) * (F32(1.0) / (F32(dx) * F32(dz)))).astype(F32)


def ricker_half_derivative(nt, dt, fcut, dx, dz):
    """The Python modeller's wavelet: Ricker filtered by sqrt(i w) in the
    frequency domain, then scaled by 1/(dx dz) (src/utils.py:21-28,
    src/Modeling2D.py:29-30)."""
    f = fcut / (3.0 * math.sqrt(math.pi))
    td = np.arange(nt) * dt - 2.0 * math.sqrt(math.pi) / fcut
    a = (math.pi * f * td) ** 2
    s = (1.0 - 2.0 * math.pi * (math.pi * f * td) * (math.pi * f * td)) * np.exp(-a * math.pi)
    w = 2.0 * math.pi * np.fft.fftfreq(nt, dt)
    s = np.real(np.fft.ifft(np.fft.fft(s) * np.sqrt(1j * w)))
    return (s / (dx * dz)).astype(F32)


def mute(seismogram, rec_x, rec_z, shot_x, shot_z, dt, v0, shift, window):
    """Zero the data before the direct arrival |r - s|/v0 + shift and taper
    linearly over `window` seconds after it; float32 as in the C++ host code
    (cpp/Migration.cu:86-115).  Only the zeroed rows and the taper rows are
    touched: searchsorted gives, per receiver, the first sample with t >= t1
    (and t >= t2) under the same float32 comparisons."""
    s = np.array(seismogram, dtype=F32, copy=True)
    nt, nrec = s.shape
    ddx = np.asarray(rec_x, F32) - F32(shot_x)
    ddz = np.asarray(rec_z, F32) - F32(shot_z)
    t1 = (np.sqrt(ddz * ddz + ddx * ddx).astype(F32) / F32(v0) + F32(shift)).astype(F32)
    t2 = (t1 + F32(window)).astype(F32)
    t = np.arange(nt, dtype=F32) * F32(dt)
    i1 = np.searchsorted(t, t1, side="left")
    i2 = np.maximum(np.searchsorted(t, t2, side="left"), i1)
    s[np.arange(nt)[:, None] < i1[None, :]] = F32(0.0)
    cols = np.arange(nrec)
    for w in range(int((i2 - i1).max()) if nrec else 0):
        rows = i1 + w
        sel = rows < i2
        r, c = rows[sel], cols[sel]
        s[r, c] = s[r, c] * ((t[r] - t1[c]) / (t2[c] - t1[c]))
    return s


def gaussian_1d(sigma):
    """Normalised 1-D Gaussian of length ceil(6 sigma + 1), made odd
    (cpp/Migration.cu:145-169): taps exp(-(x*x) / (2 sigma sigma)) rounded to
    float (the C library's expf gives the same values; numpy's float32 exp
    differs by an ulp for many of them), divided by their sum accumulated in
    order."""
    sg = F32(sigma)
    n = int(math.ceil(F32(6.0) * sg + F32(1.0)))
    if n % 2 == 0:
        n += 1
    den = F32(F32(2.0) * sg) * sg
    k = np.array([math.exp(float(F32(-(x * x)) / den)) for x in range(-(n // 2), n // 2 + 1)], dtype=F32)
    total = F32(0.0)
    for v in k:
        total = F32(total + v)
    return (k / total).astype(F32)


def smooth_model(model, sigma, parameter=False, water_model=None):
    """Separable Gaussian smoothing of slowness (velocity models) or of the
    value (anisotropy parameters, parameter=True), indices clamped at the
    edges, each tap sum accumulated in float in tap order; the cells of the
    water mask keep their value.  The mask is the cells within 1e-3 of the
    minimum of water_model, the unsmoothed velocity in the reference's use for
    every field (cpp/Migration.cu:131-143, 265-290); None: the model itself."""
    m = np.asarray(model, F32)
    w = m if water_model is None else np.asarray(water_model, F32)
    mask = np.abs(w - w.min()) < F32(1e-3)
    s0 = m.copy() if parameter else (F32(1.0) / m)
    k = gaussian_1d(sigma)
    half = k.size // 2
    nz, nx = m.shape
    pad_x = np.pad(s0, ((0, 0), (half, half)), mode="edge")
    tmp = np.zeros_like(s0)
    for i in range(k.size):
        tmp += k[i] * pad_x[:, i:i + nx]
    pad_z = np.pad(tmp, ((half, half), (0, 0)), mode="edge")
    s = np.zeros_like(s0)
    for i in range(k.size):
        s += k[i] * pad_z[i:i + nz, :]
    s = np.where(mask, s0, s).astype(F32)
    return s if parameter else (F32(1.0) / s).astype(F32)


def laplacian_filter(image, dz, dx):
    """-(d2/dz2 + d2/dx2) of the image, 2nd-order differences, edge rows and
    columns copied from their neighbours."""
    f = np.asarray(image, np.float64)
    g = np.zeros_like(f)
    g[1:-1, 1:-1] = ((f[2:, 1:-1] - 2.0 * f[1:-1, 1:-1] + f[:-2, 1:-1]) / (dz * dz)
                     + (f[1:-1, 2:] - 2.0 * f[1:-1, 1:-1] + f[1:-1, :-2]) / (dx * dx))
    g[0, :], g[-1, :] = g[1, :], g[-2, :]
    g[:, 0], g[:, -1] = g[:, 1], g[:, -2]
    return -g


def normalize_image(image, ilum, norm="cpp"):
    """Illumination normalisation of a summed image, in float32 as the engine's
    pam_rtm_result does it: "cpp" divides where the illumination exceeds
    1e-12, else 0 (cpp/Migration.cu:470-484); "py" divides by the
    illumination plus 1e-5 of its maximum (src/Migration.py:563); "none"
    returns the image.  Used where images summed over ranks are normalised
    on the host."""
    img = np.asarray(image, np.float32)
    den = np.asarray(ilum, np.float32)
    if norm == "none":
        return img.copy()
    if norm == "cpp":
        out = np.zeros_like(img)
        m = den > np.float32(1e-12)
        out[m] = img[m] / den[m]
        return out
    return (img / (den + np.float32(1e-5) * den.max())).astype(np.float32)
