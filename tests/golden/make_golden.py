"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference's own Python CPU kernels (``src/utils.py`` and the
``wavefield`` time loop of ``src/Modeling2D.py``) on small seeded grids and
stores inputs and outputs in ``tests/golden/golden_small.npz``.

The reference imports numba and cupy, which this environment does not have.
Stub modules are injected instead: ``numba.jit``/``njit`` become identity
decorators and ``prange`` becomes ``range`` (the kernels are plain Python
loops underneath), and ``cupy.RawKernel`` becomes an inert object (the GPU
kernels are never launched).  Inputs are float64, so every kernel evaluates
its formulas in float64 - the arithmetic numba would use - and the fixtures
are an FP64 evaluation of the reference formulas.

Usage (needs the reference checkout, so it runs in the development
container only; the fixtures it writes are committed):

    python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    numba = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.jit = jit
    numba.njit = jit
    numba.prange = range
    sys.modules["numba"] = numba

    cupy = types.ModuleType("cupy")

    class RawKernel:
        def __init__(self, code, name):
            self.name = name

        def __call__(self, *a, **k):
            raise RuntimeError("GPU kernels are not run by the golden generator")

    cupy.RawKernel = RawKernel
    cupy.float32 = np.float32
    cupy.asarray = np.asarray
    cupy.asnumpy = np.asarray
    sys.modules["cupy"] = cupy

    mpl = types.ModuleType("mpl_toolkits")
    ag = types.ModuleType("mpl_toolkits.axes_grid1")
    ag.make_axes_locatable = None
    mpl.axes_grid1 = ag
    sys.modules["mpl_toolkits"] = mpl
    sys.modules["mpl_toolkits.axes_grid1"] = ag


def _smooth(rng, shape, lo, hi):
    """Seeded smooth random field in [lo, hi]."""
    f = rng.standard_normal(shape)
    k = np.ones(5) / 5.0
    for ax in (0, 1):
        f = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), ax, f)
    f = (f - f.min()) / (np.ptp(f) + 1e-30)
    return lo + (hi - lo) * f


def main(ref_root):
    _install_stubs()
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import utils  # noqa: E402  (reference src/utils.py)
    import Modeling2D  # noqa: E402  (reference src/Modeling2D.py)

    rng = np.random.default_rng(20261203)
    out = {}

    # ---------------- single-kernel cases on an expanded 36 x 44 grid, N_abc = 10
    nz, nx, N = 36, 44, 10
    dz, dx, dt = 10.0, 12.0, 0.001
    vp = _smooth(rng, (nz, nx), 1500.0, 3000.0)
    eps = _smooth(rng, (nz, nx), 0.0, 0.25)
    dl = _smooth(rng, (nz, nx), 0.0, 0.1)
    th = _smooth(rng, (nz, nx), -0.6, 0.6)
    Uc = rng.standard_normal((nz, nx))
    Uf = rng.standard_normal((nz, nx))
    Uc[:4, :] = Uc[-4:, :] = 0
    Uc[:, :4] = Uc[:, -4:] = 0
    Uf[:4, :] = Uf[-4:, :] = 0
    Uf[:, :4] = Uf[:, -4:] = 0
    out.update(k_nz=nz, k_nx=nx, k_N=N, k_dz=dz, k_dx=dx, k_dt=dt,
               k_vp=vp, k_eps=eps, k_delta=dl, k_theta=th, k_Uc=Uc, k_Uf=Uf)

    out["k_acoustic"] = utils.updateWaveEquation(Uf.copy(), Uc, vp, nz, nx, dz, dx, dt)
    out["k_vti"] = utils.updateWaveEquationVTI(Uf.copy(), Uc, nx, nz, dt, dx, dz, vp, eps, dl)
    out["k_tti"] = utils.updateWaveEquationTTI(Uf.copy(), Uc, nx, nz, dt, dx, dz, vp, eps, dl, th)

    # Cerjan vector and damping (src/Modeling2D.py:258-264, src/utils.py:380-393)
    pmt = types.SimpleNamespace(N_abc=N, nz_abc=nz, nx_abc=nx, dx=dx, dz=dz, dt=dt, fcut=25.0)
    wf = Modeling2D.wavefield(pmt)
    A = wf.createCerjanVector()
    out["k_cerjanA"] = A
    out["k_damped"] = utils.AbsorbingBoundary(N, nz, nx, Uc.copy(), A)

    # CPML memory variables and updates (src/utils.py:242-377, 768-1306)
    d0, f_pico = wf.dampening_const()
    out.update(k_d0=d0, k_fpico=f_pico, k_fcut=pmt.fcut)
    PsixFR = rng.standard_normal((nz, N + 4)) * 0.01
    PsixFL = rng.standard_normal((nz, N + 4)) * 0.01
    PsizFU = rng.standard_normal((N + 4, nx)) * 0.01
    PsizFD = rng.standard_normal((N + 4, nx)) * 0.01
    ZetaxFR = rng.standard_normal((nz, N + 4)) * 0.01
    ZetaxFL = rng.standard_normal((nz, N + 4)) * 0.01
    ZetazFU = rng.standard_normal((N + 4, nx)) * 0.01
    ZetazFD = rng.standard_normal((N + 4, nx)) * 0.01
    # the reference only ever writes strip cells; entries it never writes stay zero
    for a in (PsixFL, ZetaxFL):
        a[:, :4] = 0; a[:, N:] = 0; a[:4, :] = 0; a[nz - 4:, :] = 0
    for a in (PsixFR, ZetaxFR):
        a[:, N - 4:] = 0; a[:4, :] = 0; a[nz - 4:, :] = 0
    for a in (PsizFU, ZetazFU):
        a[:4, :] = 0; a[N:, :] = 0; a[:, :4] = 0; a[:, nx - 4:] = 0
    for a in (PsizFD, ZetazFD):
        a[N - 4:, :] = 0; a[:, :4] = 0; a[:, nx - 4:] = 0
    st = dict(PsixFR=PsixFR, PsixFL=PsixFL, PsizFU=PsizFU, PsizFD=PsizFD,
              ZetaxFR=ZetaxFR, ZetaxFL=ZetaxFL, ZetazFU=ZetazFU, ZetazFD=ZetazFD)
    for k, v in st.items():
        out["k_in_" + k] = v.copy()
    pxr, pxl, pzu, pzd = utils.updatePsi(PsixFR.copy(), PsixFL.copy(), PsizFU.copy(), PsizFD.copy(),
                                         nx, nz, Uc, dx, dz, N, f_pico, d0, dt, vp)
    zxr, zxl, zzu, zzd = utils.updateZeta(pxr, pxl, ZetaxFR.copy(), ZetaxFL.copy(), pzu, pzd,
                                          ZetazFU.copy(), ZetazFD.copy(), nx, nz, Uc, dx, dz, N,
                                          f_pico, d0, dt, vp)
    out.update(k_out_PsixFR=pxr, k_out_PsixFL=pxl, k_out_PsizFU=pzu, k_out_PsizFD=pzd,
               k_out_ZetaxFR=zxr, k_out_ZetaxFL=zxl, k_out_ZetazFU=zzu, k_out_ZetazFD=zzd)
    out["k_acoustic_cpml"] = utils.updateWaveEquationCPML(Uf.copy(), Uc, vp, nx, nz, dz, dx, dt,
                                                          pxr, pxl, pzu, pzd, zxr, zxl, zzu, zzd, N)
    out["k_vti_cpml"] = utils.updateWaveEquationVTICPML(Uf.copy(), Uc, dt, dx, dz, vp, eps, dl, nx, nz,
                                                        pxr, pxl, pzu, pzd, zxr, zxl, zzu, zzd, N)

    # Adjoint (imaging) operators of the anisotropic RTM, Python CPU form
    # (src/utils.py:530-765); P is a second random field
    P = rng.standard_normal((nz, nx))
    P[:4, :] = P[-4:, :] = 0
    P[:, :4] = P[:, -4:] = 0
    out["k_P"] = P
    z = np.zeros((nz, nx))
    out["k_adj_vti"] = utils.updateAdjointWaveEquationVTI(Uf.copy(), Uc, P, z.copy(), z.copy(), z.copy(), z.copy(),
                                                          nx, nz, dt, dx, dz, vp, eps, dl)
    out["k_adj_tti"] = utils.updateAdjointWaveEquationTTI(Uf.copy(), Uc, P, z.copy(), z.copy(), z.copy(), z.copy(),
                                                          z.copy(), nx, nz, dt, dx, dz, vp, eps, dl, th)

    # Mute (src/utils.py:30-49)
    nt_m, nrec = 60, 12
    seis = rng.standard_normal((nt_m, nrec))
    rec_x = np.linspace(0.0, 550.0, nrec)
    rec_z = np.full(nrec, 20.0)
    shot_x = np.array([100.0, 300.0])
    shot_z = np.array([10.0, 10.0])
    out.update(m_seis=seis, m_rec_x=rec_x, m_rec_z=rec_z, m_shot_x=shot_x, m_shot_z=shot_z,
               m_dt=0.004, m_shift=0.02, m_window=0.03, m_v0=1500.0)
    out["m_muted"] = utils.Mute(seis, 1, rec_x, rec_z, shot_x, shot_z, 0.004, 0.02, 0.03, 1500.0)

    # Python modeller's wavelet: Ricker with a half-derivative filter (src/utils.py:21-28)
    nt_w, dt_w, f_w = 400, 0.001, 25.0
    t_w = np.arange(nt_w) * dt_w
    out.update(w_nt=nt_w, w_dt=dt_w, w_fcut=f_w,
               w_py=utils.ricker(f_w, t_w, 2.0 * np.sqrt(np.pi) / f_w, nt_w, dt_w))

    # ---------------- short full time loops through the reference wavefield driver
    # (src/Modeling2D.py:335-421), float64 arrays, C++-style (un-filtered) wavelet
    for approx in ("acoustic", "VTI", "TTI"):
        for abc in ("cerjan", "CPML"):
            if approx == "TTI" and abc == "CPML":
                continue  # the reference has no TTI CPML
            g = _run_loop(Modeling2D, rng, approx, abc)
            for k, v in g.items():
                out[f"loop_{approx}_{abc}_{k}"] = v

    # ---------------- multiparameter gradient increments (src/utils.py:1309-1463), on
    # the models above with two random fields of their own generator
    rng_mp = np.random.default_rng(4321)
    cur = rng_mp.standard_normal((nz, nx))
    adj = rng_mp.standard_normal((nz, nx))
    z = np.zeros((nz, nx))
    # calculateGradientVTI cannot run: it rebinds its `delta` array argument to a
    # scalar inside the loop (src/utils.py:1344), so the second cell fails (and
    # numba rejects the function).  At theta = 0 the TTI function's epsilon and
    # delta terms are the VTI formulas, so it gives the VTI vectors.
    ge, gd, _ = utils.calculateGradientTTI(cur, adj, z.copy(), z.copy(), z.copy(), dx, dz, nx, nz, eps, dl, z)
    ge_t, gd_t, gt_t = utils.calculateGradientTTI(cur, adj, z.copy(), z.copy(), z.copy(), dx, dz, nx, nz, eps, dl,
                                                  th)
    out.update(mp_cur=cur, mp_adj=adj, mp_vti_eps=ge, mp_vti_delta=gd, mp_tti_eps=ge_t, mp_tti_delta=gd_t,
               mp_tti_theta=gt_t)

    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)
    print("wrote", os.path.join(HERE, "golden_small.npz"), len(out), "arrays")


def _run_loop(Modeling2D, rng, approx, abc):
    nz, nx, N = 30, 38, 12
    nz_a, nx_a = nz + 2 * N, nx + 2 * N
    dz, dx, dt, fcut = 10.0, 10.0, 0.001, 30.0
    nt, itlag = 90, 10
    nt_data = nt - itlag
    vp = np.full((nz, nx), 1800.0)
    vp[nz // 2:, :] = 2600.0
    # float32-representable models, expanded in float64 below so that every
    # product is evaluated in float64 (see the module docstring)
    eps = _smooth(rng, (nz, nx), 0.02, 0.2).astype(np.float32).astype(np.float64)
    dl = _smooth(rng, (nz, nx), 0.0, 0.08).astype(np.float32).astype(np.float64)
    th = _smooth(rng, (nz, nx), -0.5, 0.5).astype(np.float32).astype(np.float64)
    rec_x = np.arange(2, nx - 2, 3) * dx
    rec_z = np.full(rec_x.size, 3 * dz)
    sx, sz = nx // 2 * dx, 2 * dz
    # C++ createWavelet (cpp/Modeling.cu:84-100) evaluated in float64
    tlag = itlag * dt
    fc = fcut / (3.0 * np.sqrt(np.pi))
    t = np.arange(nt) * dt - tlag
    arg = np.pi ** 3 * fc * fc * t * t
    src = (1.0 - 2.0 * arg) * np.exp(-arg) / (dx * dz)

    pmt = types.SimpleNamespace(
        N_abc=N, nz_abc=nz_a, nx_abc=nx_a, nz=nz, nx=nx, dx=dx, dz=dz, dt=dt, fcut=fcut,
        nt=nt, itlag=itlag, nt_data=nt_data, approximation=approx, ABC=abc, unit="CPU",
        snap=False, Nshot=1, Nrec=rec_x.size, sx=[int(round(sx / dx)) + N], sz=[int(round(sz / dz)) + N],
        rx=(np.round(rec_x / dx).astype(int) + N), rz=(np.round(rec_z / dz).astype(int) + N),
        seismogramFolder="", last_save=0, step=1)
    wf = Modeling2D.wavefield(pmt)
    # ExpandModel pads into a float32 array (src/Modeling2D.py:42); under the
    # numba stub a float32 element times a Python float would then round to
    # float32, which numba does not do.  Pad in float64 instead: the values are
    # the same (the models are float32-representable), the arithmetic is FP64.
    wf.ExpandModel = lambda m: np.pad(np.asarray(m, np.float64), N, mode="edge")
    wf.vp = vp.copy()
    wf.epsilon = eps.copy()
    wf.delta = dl.copy()
    wf.theta = th.copy()
    wf.source = src
    wf.current = np.zeros((nz_a, nx_a))
    wf.future = np.zeros((nz_a, nx_a))
    wf.seismogram = np.zeros((nt_data, pmt.Nrec))
    if abc == "CPML":
        for name, shape in (("PsixFR", (nz_a, N + 4)), ("PsixFL", (nz_a, N + 4)),
                            ("PsizFU", (N + 4, nx_a)), ("PsizFD", (N + 4, nx_a))):
            setattr(wf, name, np.zeros(shape))
            setattr(wf, name.replace("Psi", "Zeta"), np.zeros(shape))
    wf.save_seismogram = lambda shot: None  # keep the fixture run off the filesystem
    wf.reset_field = lambda: None
    wf.solveWaveEquation()
    return dict(nz=nz, nx=nx, N=N, dz=dz, dx=dx, dt=dt, fcut=fcut, nt=nt, itlag=itlag,
                vp=vp, eps=eps, delta=dl, theta=th, rx=pmt.rx, rz=pmt.rz,
                sx=pmt.sx[0], sz=pmt.sz[0], src=src, seis=wf.seismogram.copy(),
                final=wf.current.copy())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
