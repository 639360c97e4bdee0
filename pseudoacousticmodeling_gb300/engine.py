"""Python handle on the C ABI: one ``Engine`` per job configuration.

Arrays in and out are numpy float32 (host) or, for the ``*_device`` calls,
CUDA torch tensors.  Errors raise ``PamError`` with the library's message.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

MISFIT_NOALLOC_MAX_SAMPLES = 134217728   # PAM_MISFIT_NOALLOC_MAX_SAMPLES

APPROX = {"acoustic": 0, "VTI": 1, "TTI": 2}
BOUNDARY = {"cerjan": 0, "CPML": 1}
STORE = {"f32": 0, "bf16": 1, "f16": 2}
BOUNDARY_SAVING = -1    # ckpt_interval value: rebuild the source field from saved boundary bands
RANDOM_BOUNDARY = -2    # ckpt_interval value: undamped source field through a random border, run backwards
NORM = {"none": 0, "cpp": 1, "py": 2}


@dataclass
class Config:
    """One job: interior grid, absorbing width, time axis and operator."""
    nz: int
    nx: int
    n_abc: int
    dz: float
    dx: float
    dt: float
    nt: int
    itlag: int
    fcut: float
    approximation: str = "acoustic"
    boundary: str = "cerjan"
    max_shots: int = 1

    @property
    def nt_data(self):
        return self.nt - self.itlag

    @property
    def nz_abc(self):
        return self.nz + 2 * self.n_abc

    @property
    def nx_abc(self):
        return self.nx + 2 * self.n_abc

    def to_c(self):
        return _lib.PamConfig(self.nz, self.nx, self.n_abc, self.dz, self.dx, self.dt, self.nt, self.itlag,
                              self.fcut, APPROX[self.approximation], BOUNDARY[self.boundary], self.max_shots)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Engine:
    def __init__(self, cfg: Config, device: int = 0):
        self.lib = _lib.load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        c = cfg.to_c()
        rc = self.lib.pam_create(ctypes.byref(c), device, ctypes.byref(h))
        self.h = h
        if rc != _lib.PAM_OK:
            msg = self.lib.pam_last_error(h).decode() if h.value else "pam_create failed"
            self.close()
            raise _lib.PamError(rc, msg)
        self.nrec = 0
        nz, nx, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.pam_grid_info(self.h, ctypes.byref(nz), ctypes.byref(nx), ctypes.byref(p))
        self.pitch = p.value

    def _check(self, rc):
        if rc < 0:
            raise _lib.PamError(rc, self.lib.pam_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.pam_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ setup
    def set_models(self, vp, eps=None, delta=None, theta_deg=None):
        self._keep = [_f32(vp), None if eps is None else _f32(eps), None if delta is None else _f32(delta),
                      None if theta_deg is None else _f32(theta_deg)]
        self._check(self.lib.pam_set_models(self.h, *[_ptr(a) for a in self._keep]))

    def set_wavelet(self, w):
        w = _f32(w)
        self._check(self.lib.pam_set_wavelet(self.h, _ptr(w)))

    def set_damping(self, factors):
        """Cerjan damping factors [n_abc] (index 0 at the outer edge); ones
        make the border undamped (pam_set_damping)."""
        f = _f32(factors)
        self._check(self.lib.pam_set_damping(self.h, _ptr(f)))

    def set_receivers(self, rz, rx, per_shot=False):
        rz, rx = _i32(rz), _i32(rx)
        n = rz.shape[-1]
        self._check(self.lib.pam_set_receivers(self.h, n, _ptr(rz), _ptr(rx), 1 if per_shot else 0))
        self.nrec = n

    def field_bytes(self):
        """Bytes of one shot's wavefield on the device (expanded grid, row pitch)."""
        return self.cfg.nz_abc * self.pitch * 4

    def plan_checkpoints(self, budget_bytes, store="f32"):
        """(ckpt_interval, recomputed steps) of the checkpoint plan with the
        fewest recomputed steps whose buffers fit in budget_bytes
        (pam_plan_checkpoints); ckpt_interval 0 stores every step."""
        k, rec = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.pam_plan_checkpoints(self.h, int(budget_bytes), STORE[store], ctypes.byref(k),
                                                  ctypes.byref(rec)))
        return k.value, rec.value

    def check_stability(self):
        dt, dx = ctypes.c_float(), ctypes.c_float()
        ok = self._check(self.lib.pam_check_stability(self.h, ctypes.byref(dt), ctypes.byref(dx)))
        return bool(ok), dt.value, dx.value

    # ------------------------------------------------------------ modelling
    def forward(self, sz, sx, out=None, stream=None):
        """Host path: model the shots at (sz, sx) and return their seismograms
        [n][nt_data][nrec] (written into `out` when given; pinned memory makes
        the copy back fastest).  `stream`: a CUDA stream handle (None: the
        engine's own stream)."""
        sz, sx = _i32(sz), _i32(sx)
        n = sz.size
        if out is None:
            out = np.empty((n, self.cfg.nt_data, self.nrec), np.float32)
        self._check(self.lib.pam_forward(self.h, n, _ptr(sz), _ptr(sx), _ptr(out),
                                         None if stream is None else ctypes.c_void_p(stream)))
        return out

    def forward_device(self, d_sz, d_sx, d_seis, stream=None):
        """Device path: int32 CUDA tensors sz, sx [n]; float32 CUDA tensor seis [n][nt_data][nrec]."""
        n = d_sz.numel()
        self._check(self.lib.pam_forward_device(self.h, n, ctypes.c_void_p(d_sz.data_ptr()),
                                                ctypes.c_void_p(d_sx.data_ptr()),
                                                ctypes.c_void_p(d_seis.data_ptr()),
                                                None if stream is None else ctypes.c_void_p(stream)))

    def misfit_device(self, d_dcal, d_dobs, stream=None):
        """0.5 sum (dcal - dobs)^2 of two float32 CUDA tensors of equal size,
        reduced on the GPU (pam_misfit_noalloc, in pieces of at most
        MISFIT_NOALLOC_MAX_SAMPLES samples); waits for `stream`."""
        n = d_dcal.numel()
        if d_dobs.numel() != n:
            raise ValueError("dcal and dobs differ in size")
        a, b = d_dcal.reshape(-1), d_dobs.reshape(-1)
        total = 0.0
        part = ctypes.c_double(0.0)
        for i0 in range(0, n, MISFIT_NOALLOC_MAX_SAMPLES):
            m = min(MISFIT_NOALLOC_MAX_SAMPLES, n - i0)
            self._check(self.lib.pam_misfit_noalloc(ctypes.c_void_p(a[i0:].data_ptr()),
                                                    ctypes.c_void_p(b[i0:].data_ptr()), m, ctypes.byref(part),
                                                    None if stream is None else ctypes.c_void_p(stream)))
            total += part.value
        return total

    def begin(self, sz, sx):
        sz, sx = _i32(sz), _i32(sx)
        self._nsteps_shots = sz.size
        self._check(self.lib.pam_begin(self.h, sz.size, _ptr(sz), _ptr(sx)))

    def step(self, k):
        self._check(self.lib.pam_step(self.h, k))

    def read_seismograms(self):
        out = np.empty((self._nsteps_shots, self.cfg.nt_data, self.nrec), np.float32)
        self._check(self.lib.pam_read_seismograms(self.h, _ptr(out)))
        return out

    def read_wavefield(self, shot=0):
        out = np.empty((self.cfg.nz_abc, self.cfg.nx_abc), np.float32)
        self._check(self.lib.pam_read_wavefield(self.h, shot, _ptr(out)))
        return out

    def profile(self, stride):
        """Sample every `stride`-th step's kernels with CUDA events (0 = off)."""
        self._check(self.lib.pam_profile_enable(self.h, int(stride)))

    def set_random_boundary(self, dvel=1000.0, ratio=200.0, seed=0):
        """Parameters of the random border used with ckpt_interval=RANDOM_BOUNDARY."""
        self._check(self.lib.pam_set_random_boundary(self.h, float(dvel), float(ratio), int(seed)))

    def autotune(self, enable=True):
        """Turn the stepping kernel's segment-height tuner on or off."""
        self._check(self.lib.pam_autotune(self.h, 1 if enable else 0))

    def segment_height(self, nshots):
        """Segment height chosen for a batch of `nshots` (0: not tuned yet)."""
        return int(self.lib.pam_segment_height(self.h, int(nshots)))

    def profile_read(self):
        """{class: (total ms, sampled launches)} of the last completed run:
        the forward steps' stepping, CPML-strip and recording kernels, and the
        backward steps' receiver-side adjoint kernel and imaging / gradient sum."""
        names = ("step", "cpml", "record", "adjoint", "imaging")
        ms = (ctypes.c_double * len(names))()
        cnt = (ctypes.c_int * len(names))()
        self._check(self.lib.pam_profile_read(self.h, ms, cnt, len(names)))
        return {names[i]: (ms[i], cnt[i]) for i in range(len(names))}

    # ------------------------------------------------------------ migration / inversion
    def rtm(self, sz, sx, dobs, ckpt_interval=0, store="f32"):
        sz, sx, d = _i32(sz), _i32(sx), _f32(dobs)
        self._check(self.lib.pam_rtm(self.h, sz.size, _ptr(sz), _ptr(sx), _ptr(d), int(ckpt_interval),
                                     STORE[store], None))

    def rtm_result(self, norm="cpp"):
        img = np.empty((self.cfg.nz, self.cfg.nx), np.float32)
        ilum = np.empty((self.cfg.nz, self.cfg.nx), np.float32)
        self._check(self.lib.pam_rtm_result(self.h, _ptr(img), _ptr(ilum), NORM[norm]))
        return img, ilum

    def set_mute(self, shot_x, shot_z, rec_x, rec_z, v0, shift, window):
        """Arm the GPU mute of the observed data (cpp/Migration.cu:86-115) for
        the next rtm call, whose shots are the len(shot_x) given here:
        coordinates in metres, rec_x/rec_z [nrec] or [shots][nrec] per shot."""
        sxa, sza = _f32(np.ravel(shot_x)), _f32(np.ravel(shot_z))
        rxa, rza = _f32(rec_x), _f32(rec_z)
        per_shot = rxa.ndim == 2
        nrec = rxa.shape[-1]
        self._check(self.lib.pam_set_mute(self.h, sxa.size, _ptr(sxa), _ptr(sza), nrec, _ptr(rxa), _ptr(rza),
                                          1 if per_shot else 0, float(v0), float(shift), float(window)))

    def clear_mute(self):
        self._check(self.lib.pam_set_mute(self.h, 0, None, None, 0, None, None, 0, 1.0, 0.0, 0.0))

    def rtm_reset(self):
        self._check(self.lib.pam_rtm_reset(self.h))

    def fwi_gradient(self, sz, sx, dobs, ckpt_interval=0, store="f32"):
        sz, sx, d = _i32(sz), _i32(sx), _f32(dobs)
        mis = ctypes.c_double(0.0)
        self._check(self.lib.pam_fwi_gradient(self.h, sz.size, _ptr(sz), _ptr(sx), _ptr(d), int(ckpt_interval),
                                              STORE[store], ctypes.byref(mis), None))
        return mis.value

    def fwi_result(self):
        g = np.empty((self.cfg.nz, self.cfg.nx), np.float32)
        ilum = np.empty((self.cfg.nz, self.cfg.nx), np.float32)
        self._check(self.lib.pam_fwi_result(self.h, _ptr(g), _ptr(ilum)))
        return g, ilum

    def set_multiparameter(self, enable=True):
        """Also accumulate the epsilon, delta (theta) gradients in fwi_gradient (VTI/TTI)."""
        self._check(self.lib.pam_set_multiparameter(self.h, 1 if enable else 0))

    def fwi_multiparameter_result(self):
        """(g_eps, g_delta, g_theta or None) [nz][nx], un-normalised."""
        shp = (self.cfg.nz, self.cfg.nx)
        ge, gd = np.empty(shp, np.float32), np.empty(shp, np.float32)
        gt = np.empty(shp, np.float32) if self.cfg.approximation == "TTI" else None
        self._check(self.lib.pam_fwi_multiparameter_result(self.h, _ptr(ge), _ptr(gd),
                                                           None if gt is None else _ptr(gt)))
        return ge, gd, gt

    def misfit_gradient(self, sz, sx, dobs, ckpt_interval=0, store="f32"):
        """Exact L2 misfit and its gradient with respect to vp [nz][nx]."""
        sz, sx, d = _i32(sz), _i32(sx), _f32(dobs)
        mis = ctypes.c_double(0.0)
        g = np.zeros((self.cfg.nz, self.cfg.nx), np.float32)
        self._check(self.lib.pam_misfit_gradient(self.h, sz.size, _ptr(sz), _ptr(sx), _ptr(d), int(ckpt_interval),
                                                 STORE[store], ctypes.byref(mis), _ptr(g), None))
        return mis.value, g

    def adjoint_gradient(self, sz, sx, adjoint_source, ckpt_interval=0, store="f32"):
        """(dF/dvp)^T adjoint_source [nz][nx] for the forward map d = F(vp) of
        the shots (sz, sx): the exact adjoint applied to adjoint_source
        [n][nt_data][nrec] itself (pam_adjoint_gradient)."""
        sz, sx, a = _i32(sz), _i32(sx), _f32(adjoint_source)
        g = np.zeros((self.cfg.nz, self.cfg.nx), np.float32)
        self._check(self.lib.pam_adjoint_gradient(self.h, sz.size, _ptr(sz), _ptr(sx), _ptr(a), int(ckpt_interval),
                                                  STORE[store], _ptr(g), None))
        return g


def smooth_model(model, sigma, parameter=False, water_model=None):
    """Migration model smoothing (cpp/Migration.cu:131-236) on the GPU through
    pam_smooth_model; returns a new float32 [nz][nx] array.  water_model is
    the unsmoothed velocity whose minimum marks the water layer (the
    reference's mask for every smoothed field); None: the model itself."""
    out = np.array(model, dtype=np.float32, copy=True, order="C")
    w = None
    if water_model is not None:
        w = np.ascontiguousarray(water_model, dtype=np.float32)
        if w.shape != out.shape:
            raise ValueError(f"water_model has shape {w.shape}, the model {out.shape}")
    rc = _lib.load().pam_smooth_model(_ptr(out), out.shape[0], out.shape[1], float(sigma), 1 if parameter else 0,
                                      _ptr(w))
    if rc != 0:
        raise _lib.PamError(rc, "pam_smooth_model failed")
    return out


def laplacian_filter_gpu(image, dz, dx):
    """-(d2/dz2 + d2/dx2) of an image [nz][nx] on the GPU
    (pam_laplacian_filter, src/Viewdata.py:23-41); returns float32."""
    img = _f32(image)
    out = np.empty_like(img)
    rc = _lib.load().pam_laplacian_filter(_ptr(img), img.shape[0], img.shape[1], float(dz), float(dx), _ptr(out))
    if rc != 0:
        raise _lib.PamError(rc, "pam_laplacian_filter failed")
    return out
