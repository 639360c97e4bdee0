"""Host layer: the reference's job files and the preparation steps (no GPU)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from pseudoacousticmodeling_gb300 import preprocess
from pseudoacousticmodeling_gb300.survey import import_bin, parameters, save_bin, write_csv_geometry


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _job(tmp_path, **over):
    p = {"unit": "GPU", "approximation": "VTI", "migration": "checkpoint", "ABC": "CPML", "dx": 10.0, "dz": 10.0,
         "dt": 0.0008, "L": 20000.0, "D": 8000.0, "T": 3.1992, "N_abc": 50, "fcut": 12.0,
         "rec_file": "rec.csv", "src_file": "src.csv", "seismogramFolder": "out/"}
    p.update(over)
    path = tmp_path / "Parameters.json"
    path.write_text(json.dumps(p))
    write_csv_geometry(tmp_path / "rec.csv", np.arange(0, 20001, 10.0), np.full(2001, 10.0))
    write_csv_geometry(tmp_path / "src.csv", 150.0 * np.arange(128), np.full(128, 10.0))
    return path


def test_parameters_cpp_and_python_rounding(tmp_path):
    path = _job(tmp_path)
    c = parameters(str(path))
    py = parameters(str(path), rounding="python")
    # C++ rounds (cpp/Survey.cpp:101-108); Python truncates (src/survey.py:41-44)
    assert (c.nz, c.nx, c.N_abc) == (801, 2001, 50)
    assert c.itlag == 369 and c.nt_data == 4000 and c.nt == 4369
    assert py.nt_data == 3999      # int(3.1992 / 0.0008) = 3998 + 1
    assert c.nz_abc == 901 and c.nx_abc == 2101
    assert c.Nrec == 2001 and c.Nshot == 128
    assert c.rx[0] == 50 and c.rx[-1] == 2050 and (c.rz == 51).all()
    assert c.sx[1] == 65 and (c.sz == 51).all()
    assert c.seismogram_file(0).endswith("seismogram_shot_1_Nt4000_Nrec2001_fcut12.0.bin")
    cfg = c.engine_config(max_shots=16)
    assert (cfg.nz, cfg.nx, cfg.nt, cfg.itlag, cfg.approximation, cfg.boundary) == (801, 2001, 4369, 369, "VTI",
                                                                                       "CPML")


def test_parameters_source_field_strategy_and_bands(tmp_path):
    c = parameters(str(_job(tmp_path)))                       # "checkpoint", no ckpt_interval: the reference's step
    assert c.source_field_interval == c.step
    assert parameters(str(_job(tmp_path, ckpt_interval=40))).source_field_interval == 40
    assert parameters(str(_job(tmp_path, migration="onthefly"))).source_field_interval == 0
    assert parameters(str(_job(tmp_path, migration="SB"))).source_field_interval == -1
    assert parameters(str(_job(tmp_path, migration="RBC"))).source_field_interval == -2
    with pytest.raises(ValueError, match="migration"):
        parameters(str(_job(tmp_path, migration="full")))
    # a lower cutoff frequency: longer wavelet lag, more steps (src/Inversion.py:285-296)
    cfg = c.engine_config(fcut=6.0)
    assert cfg.itlag == 739 and cfg.nt == 739 + 4000 and cfg.fcut == 6.0
    assert c.lag_steps(12.0) == c.itlag


def test_parameters_reciprocity_and_mirror(tmp_path):
    path = _job(tmp_path, reciprocity=True, mirror=True, idx_water=5)
    c = parameters(str(path))
    assert c.Nrec == 128 and c.Nshot == 2001          # sources and receivers swapped
    assert (c.rz == 51 - 5).all() and (c.sz == 51 - 5).all()


def test_parameters_errors(tmp_path):
    path = _job(tmp_path)
    d = json.loads(path.read_text())
    del d["fcut"]
    path.write_text(json.dumps(d))
    with pytest.raises(ValueError, match="fcut"):
        parameters(str(path))
    path = _job(tmp_path, approximation="elastic")
    with pytest.raises(ValueError, match="approximation"):
        parameters(str(path))
    with pytest.raises(ValueError, match="Could not open"):
        import_bin(str(tmp_path / "missing.bin"), (3, 4))
    save_bin(str(tmp_path / "short.bin"), np.zeros(5))
    with pytest.raises(ValueError, match="5 floats"):
        import_bin(str(tmp_path / "short.bin"), (3, 4))


def test_wavelets(golden):
    G = golden
    w = preprocess.ricker(300, 0.001, 15.0, 10.0, 10.0)
    ref = O.ricker_cpp(300, 0.001, 15.0, np.float32(2.0) * np.sqrt(np.float32(np.pi), dtype=np.float32)
                       / np.float32(15.0), 10.0, 10.0)
    assert rel(w, ref) < 1e-6
    wp = preprocess.ricker_half_derivative(int(G["w_nt"]), float(G["w_dt"]), float(G["w_fcut"]), 1.0, 1.0)
    assert rel(wp, G["w_py"]) < 1e-6


def test_mute_matches_reference(golden):
    G = golden
    got = preprocess.mute(G["m_seis"], G["m_rec_x"], G["m_rec_z"], G["m_shot_x"][1], G["m_shot_z"][1],
                          float(G["m_dt"]), float(G["m_v0"]), float(G["m_shift"]), float(G["m_window"]))
    assert rel(got, G["m_muted"]) < 1e-6


def _golden_host():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_host.npz"))


def test_smoothing_equals_the_reference_golden():
    """The oracle's and the package's restatements of Migration::createMask /
    smoothModel (cpp/Migration.cu:131-236) equal the reference's own compiled
    smoothing bit for bit (tests/golden/golden_host.npz, made by
    tests/golden/make_golden_host.py), every field with the water mask of the
    unsmoothed velocity as Migration::setModel uses it (cpp/Migration.cu:265-290)."""
    G = _golden_host()
    n = 0
    for c in G["smooth_cases"]:
        name, field, sigma, parameter = str(c).split("|")
        f, want = G[f"in_{field}"], G[f"out_{name}"]
        par = parameter == "1"
        np.testing.assert_array_equal(O.smooth_model_cpp(f, float(sigma), par, water_model=G["in_vp"]), want, name)
        np.testing.assert_array_equal(preprocess.smooth_model(f, float(sigma), par, water_model=G["in_vp"]), want,
                                      name)
        n += 1
    assert n == 7
    # the water layer (the velocity's minimum) is kept; eps's own zero below it is smoothed
    assert (G["out_vp_s4.5"][:9] == G["in_vp"][:9]).all()
    assert G["out_eps_s3.0"][20, 5] > 0.0
    assert O.smooth_model_cpp(G["in_eps"], 3.0, True)[20, 5] == 0.0     # what eps's own mask would keep


def test_mute_equals_the_reference_golden():
    """preprocess.mute (the host restatement the GPU mute kernel is held to
    bit for bit) and the oracle's mute equal the reference's compiled
    Migration::Mute (cpp/Migration.cu:86-115) bit for bit."""
    G = _golden_host()
    for c in G["mute_cases"]:
        name, nt, nrec, dt, v0, shift, window, sx, sz = str(c).split("|")
        seis, rx, rz = G[f"{name}_in"], G[f"{name}_rx"], G[f"{name}_rz"]
        want = G[f"{name}_out"]
        assert want.shape == (int(nt), int(nrec))
        got = preprocess.mute(seis, rx, rz, float(sx), float(sz), float(dt), float(v0), float(shift), float(window))
        np.testing.assert_array_equal(got, want, name)
        got = O.mute(seis, rx, rz, float(sx), float(sz), float(dt), float(shift), float(window), float(v0))
        np.testing.assert_array_equal(got, want, name)
        assert (want == 0.0).any() and (want == seis).any()


def test_stability_limits_equal_the_reference_golden():
    """pam_stability_limits (engine-free C ABI entry) returns exactly the
    critical dt and dx that the reference's compiled
    Modeling::checkDispersionAndStability (cpp/Modeling.cu:184-327) reports
    (dz's limit is dx's there), and the same verdict, for acoustic, VTI and TTI
    models including two that fail the check."""
    import ctypes
    from pseudoacousticmodeling_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    G = _golden_host()
    ptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
    for c in G["stability_cases"]:
        name, approx, dx, dz, dt, fcut = str(c).split("|")
        a = {"acoustic": 0, "VTI": 1, "TTI": 2}[approx]
        arrs = [G["in_vp"], G["in_eps"] if a else None, G["in_delta"] if a else None, G["in_theta"] if a == 2 else None]
        dt_lim, dx_lim = ctypes.c_float(), ctypes.c_float()
        rc = lib.pam_stability_limits(a, 37, 53, *[ptr(v) for v in arrs], float(dx), float(dz), float(dt), float(fcut),
                                      ctypes.byref(dt_lim), ctypes.byref(dx_lim))
        want = G[f"{name}_limits"]
        assert np.float32(dt_lim.value) == want[0] and np.float32(dx_lim.value) == want[1] == want[2], name
        assert rc == int(bool(G[f"{name}_satisfied"])), name


def test_padding_equals_the_reference_golden():
    """The oracle's edge-replicating padding (the expanded models of every
    oracle run) equals the reference's compiled Modeling::expandModel
    (cpp/Modeling.cu:130-182) bit for bit."""
    G = _golden_host()
    np.testing.assert_array_equal(O.expand_model(G["in_vp"], 50), G["pad_vp_N50"])
    np.testing.assert_array_equal(O.expand_model(G["in_theta"], 8), G["pad_theta_N8"])


def test_host_routines_against_the_reference_build():
    """Where the reference sources were present at build time, its compiled
    host routines (oracle/ref_host.cpp around cpp/Migration.cu and
    cpp/Modeling.cu) against the restatements on seeded shapes, bit for bit:
    smoothing, mute, stability limits, padding."""
    import ctypes
    from oracle import ref as R
    if R.host_lib() is None:
        pytest.skip("the reference's host routines were not built here (reference sources absent)")
    from pseudoacousticmodeling_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    rng = np.random.default_rng(11)
    for nz, nx, sigma in [(1, 9, 1.3), (17, 4, 2.2), (40, 61, 5.0), (64, 33, 0.4), (25, 25, 30.0)]:
        vp = (1500.0 + 2000.0 * rng.random((nz, nx))).astype(np.float32)
        vp[: nz // 4] = 1450.0
        eps = (0.3 * rng.random((nz, nx))).astype(np.float32)
        dl = (0.15 * rng.random((nz, nx))).astype(np.float32)
        th = (-40.0 + 80.0 * rng.random((nz, nx))).astype(np.float32)
        for f, par in ((vp, False), (eps, True)):
            np.testing.assert_array_equal(R.smooth_model(f, sigma, par, water_model=vp),
                                          O.smooth_model_cpp(f, sigma, par, water_model=vp), f"{nz}x{nx} {sigma}")
        for a, name, arrs in ((0, "acoustic", (vp,)), (1, "VTI", (vp, eps, dl)), (2, "TTI", (vp, eps, dl, th))):
            r = R.stability(name, *arrs, dx=7.0, dz=9.0, dt=7e-4, fcut=15.0)
            keep = list(arrs) + [None] * (4 - len(arrs))
            d1, d2 = ctypes.c_float(), ctypes.c_float()
            rc = lib.pam_stability_limits(a, nz, nx, *[None if v is None else v.ctypes.data_as(ctypes.c_void_p)
                                                       for v in keep], 7.0, 9.0, 7e-4, 15.0, ctypes.byref(d1),
                                          ctypes.byref(d2))
            assert (np.float32(d1.value), np.float32(d2.value), rc) == (r["dt_lim"], r["dx_lim"], int(r["satisfied"]))
    for nz, nx, N in [(5, 7, 3), (1, 1, 8), (40, 61, 50)]:
        f = rng.random((nz, nx)).astype(np.float32)
        np.testing.assert_array_equal(R.expand_model(f, N), O.expand_model(f, N))
    for nt, nrec, dt in [(200, 33, 0.002), (57, 5, 0.0007)]:
        seis = rng.standard_normal((nt, nrec)).astype(np.float32)
        rx = (4000.0 * rng.random(nrec)).astype(np.float32)
        rz = (50.0 * rng.random(nrec)).astype(np.float32)
        np.testing.assert_array_equal(R.mute(seis, rx, rz, 1500.0, 12.0, dt, 1500.0, 0.05, 0.04),
                                      preprocess.mute(seis, rx, rz, 1500.0, 12.0, dt, 1500.0, 0.05, 0.04))


def test_laplacian_matches_oracle():
    rng = np.random.default_rng(3)
    img = rng.standard_normal((40, 50))
    assert rel(preprocess.laplacian_filter(img, 5.0, 5.0), O.laplacian_filter(img, 5.0, 5.0)) < 1e-12


def test_shard_covers_every_shot_once():
    from pseudoacousticmodeling_gb300.distributed import shard
    for n in (1, 7, 128, 200):
        for w in (1, 2, 3, 8):
            parts = [shard(n, r, w) for r in range(w)]
            assert np.array_equal(np.concatenate(parts), np.arange(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_lbfgs_two_loop_recursion_numpy_and_torch():
    """The L-BFGS direction (src/Inversion.py:88-123) is the same on numpy
    arrays and torch tensors, and the implied inverse Hessian satisfies the
    secant condition of the newest pair (H y = s)."""
    torch = pytest.importorskip("torch")
    from pseudoacousticmodeling_gb300.inversion import two_loop_recursion
    rng = np.random.default_rng(3)
    n = 40
    H = np.diag(rng.uniform(1.0, 4.0, n))                 # Hessian of a separable quadratic
    S = [rng.normal(size=n) for _ in range(8)]
    Y = [H @ s for s in S]
    g = rng.normal(size=n)
    r_np = two_loop_recursion(g, S, Y)
    r_t = two_loop_recursion(torch.tensor(g), [torch.tensor(s) for s in S], [torch.tensor(y) for y in Y])
    assert np.allclose(r_np, r_t.numpy(), rtol=1e-12, atol=1e-12)
    assert np.allclose(two_loop_recursion(Y[-1], S, Y), S[-1], rtol=1e-9, atol=1e-9)
    assert np.array_equal(two_loop_recursion(g, [], []), g)   # no history: steepest descent


def test_misfit_device_splits_at_the_sample_limit(monkeypatch):
    """Engine.misfit_device calls pam_misfit_noalloc on pieces of at most
    MISFIT_NOALLOC_MAX_SAMPLES samples and sums their misfits (host logic,
    with a stand-in for the library)."""
    torch = pytest.importorskip("torch")
    import ctypes
    from pseudoacousticmodeling_gb300 import engine as E
    monkeypatch.setattr(E, "MISFIT_NOALLOC_MAX_SAMPLES", 7)
    calls = []

    class FakeLib:
        def pam_misfit_noalloc(self, pa, pb, n, out, stream):
            a = np.ctypeslib.as_array(ctypes.cast(pa, ctypes.POINTER(ctypes.c_float)), shape=(n,))
            b = np.ctypeslib.as_array(ctypes.cast(pb, ctypes.POINTER(ctypes.c_float)), shape=(n,))
            calls.append(n)
            out._obj.value = 0.5 * float(np.sum((a.astype(np.float64) - b) ** 2))
            return 0

    e = E.Engine.__new__(E.Engine)
    e.lib = FakeLib()
    e.h = None
    a = torch.arange(30, dtype=torch.float32).reshape(2, 15)
    b = torch.full((2, 15), 3.0)
    assert e.misfit_device(a, b) == pytest.approx(0.5 * float(((a.double() - 3.0) ** 2).sum()))
    assert calls == [7, 7, 7, 7, 2]
    with pytest.raises(ValueError):
        e.misfit_device(a, b[:1])


def test_lbfgs_converges_on_rosenbrock():
    """The reference's optimiser toy (src/optimazation.py:4-180): L-BFGS with
    the package's two-loop recursion and a strong-Wolfe line search minimises
    the Rosenbrock function from (-1.2, 1) to (1, 1)."""
    from scipy.optimize import line_search
    from pseudoacousticmodeling_gb300.inversion import two_loop_recursion

    def f(p):
        return (1.0 - p[0]) ** 2 + 100.0 * (p[1] - p[0] ** 2) ** 2

    def grad(p):
        return np.array([-2.0 * (1.0 - p[0]) - 400.0 * p[0] * (p[1] - p[0] ** 2), 200.0 * (p[1] - p[0] ** 2)])

    x = np.array([-1.2, 1.0])
    g = grad(x)
    S, Y = [], []
    for it in range(100):
        p = -two_loop_recursion(g, S, Y)
        if float(g @ p) >= 0.0:            # not a descent direction: restart
            S, Y, p = [], [], -g
        alpha = line_search(f, grad, x, p, gfk=g)[0]
        if alpha is None:                  # no Wolfe point along p: steepest descent, small step
            S, Y, p, alpha = [], [], -g, 1e-3
        x_new = x + alpha * p
        g_new = grad(x_new)
        s, y = x_new - x, g_new - g
        if float(s @ y) > 1e-12:
            S.append(s)
            Y.append(y)
            if len(S) > 8:
                S.pop(0)
                Y.pop(0)
        x, g = x_new, g_new
        if np.linalg.norm(g) < 1e-8:
            break
    assert np.allclose(x, [1.0, 1.0], atol=1e-6)


class _QuadraticEngine:
    """Stand-in for Engine in the FWI loop: its 'seismograms' are the velocities
    themselves, so the misfit is 0.5 |vp - vp_true|^2 with gradient vp - vp_true
    (flat illumination)."""

    def __init__(self, vtrue):
        self.vtrue = np.asarray(vtrue, np.float64)
        self.vp = None

    def set_models(self, vp):
        self.vp = np.asarray(vp, np.float64)

    def forward(self, sz, sx):
        return self.vp.reshape(1, 1, -1).astype(np.float32)

    def rtm_reset(self):
        pass

    def misfit_gradient(self, sz, sx, dobs, ckpt_interval=0, store="f32"):
        r = self.vp - self.vtrue
        return 0.5 * float((r * r).sum()), r.astype(np.float32)

    def fwi_result(self):
        return None, np.ones(self.vp.shape, np.float32)


def test_fwi_loop_resumes_from_its_checkpoint(tmp_path):
    """The L-BFGS loop of inversion.fwi (src/Inversion.py:290-411), driven by a
    stand-in engine on the host: the misfit falls, the model stays inside the
    velocity bounds, and a run stopped after two iterations and resumed from
    its checkpoint file ends bitwise where an uninterrupted run ends."""
    from pseudoacousticmodeling_gb300.inversion import fwi
    rng = np.random.default_rng(5)
    vtrue = rng.uniform(1800.0, 2600.0, (6, 7)).astype(np.float32)
    v0 = np.full_like(vtrue, 2200.0)

    def run(niter, checkpoint=None):
        inv = fwi(_QuadraticEngine(vtrue), [0], [0], vtrue.reshape(1, 1, -1), vmin=1500.0, vmax=3000.0,
                  device="cpu")
        return inv.solveFullWaveformInversion(v0, niter=niter, checkpoint=checkpoint), inv.history

    full, h_full = run(5)
    # the reference's step control moves m by at most 1% of its largest value
    # per iteration (src/Inversion.py:125-193), so the misfit falls slowly
    assert h_full[-1] < 0.9 * h_full[0] and h_full == sorted(h_full, reverse=True)
    assert full.min() >= 1500.0 - 1e-3 and full.max() <= 3000.0 + 1e-3
    ck = str(tmp_path / "fwi_state.npz")
    _, h_two = run(2, ck)
    assert h_two == h_full[:3]
    resumed, h_res = run(5, ck)
    assert np.array_equal(resumed, full) and h_res == h_full


def test_fwi_resume_refuses_a_state_of_another_problem(tmp_path):
    """A saved loop state is resumed only by the problem that wrote it: other
    observed data, another model shape or another L-BFGS memory raise
    ValueError instead of continuing a stale run."""
    import pytest
    from pseudoacousticmodeling_gb300.inversion import fwi
    rng = np.random.default_rng(6)
    vtrue = rng.uniform(1800.0, 2600.0, (6, 7)).astype(np.float32)
    v0 = np.full_like(vtrue, 2200.0)
    ck = str(tmp_path / "state.npz")

    def make(vt, dobs):
        return fwi(_QuadraticEngine(vt), [0], [0], dobs, vmin=1500.0, vmax=3000.0, device="cpu")

    make(vtrue, vtrue.reshape(1, 1, -1)).solveFullWaveformInversion(v0, niter=2, checkpoint=ck)
    # same problem: resumes
    make(vtrue, vtrue.reshape(1, 1, -1)).solveFullWaveformInversion(v0, niter=3, checkpoint=ck)
    # other observed data
    with pytest.raises(ValueError, match="another problem"):
        make(vtrue, (vtrue + 1.0).reshape(1, 1, -1)).solveFullWaveformInversion(v0, niter=4, checkpoint=ck)
    # other L-BFGS memory
    with pytest.raises(ValueError, match="key_memory"):
        make(vtrue, vtrue.reshape(1, 1, -1)).solveFullWaveformInversion(v0, niter=4, memory=3, checkpoint=ck)
    # other model shape
    v2 = rng.uniform(1800.0, 2600.0, (5, 7)).astype(np.float32)
    with pytest.raises(ValueError):
        make(v2, vtrue.reshape(1, 1, -1)).solveFullWaveformInversion(np.full_like(v2, 2200.0), niter=4,
                                                                      checkpoint=ck)
