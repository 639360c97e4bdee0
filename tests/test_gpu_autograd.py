"""The differentiable modelling operator and the FWI driver on the GPU.

The gradient of an L2 misfit taken through torch autograd (Propagate, whose
backward is the engine's exact adjoint) is checked against central finite
differences of the FP64 oracle's misfit at 32 random interior cells, and
against the one-call L2Misfit.  A short L-BFGS run of the reference driver
must lower the misfit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import engine_for, make_case, oracle_models, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


def _problem(seed=12):
    case = make_case("acoustic", "cerjan", nz=40, nx=90, N=20, nt=320, nshots=2, seed=seed)
    g = case["grid"]
    true = case["vp"].copy()
    zc = g.nz // 4
    true[zc - 3:zc + 3, g.nx // 2 - 8:g.nx // 2 + 8] += 250.0
    c2 = dict(case)
    c2["vp"] = true
    mt = oracle_models(c2)
    dobs = np.stack([O.forward_shot(g, mt, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"],
                                    dtype=np.float64) for sx, sz in zip(case["sx"], case["sz"])]).astype(np.float32)
    return case, dobs


def _oracle_misfit(case, vp, dobs):
    g = case["grid"]
    c = dict(case)
    c["vp"] = vp
    m = oracle_models(c)
    m = O.Models(vp=O.expand_model(np.asarray(vp, np.float64), g.N), A=m.A.astype(np.float64))
    J = 0.0
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        d = O.forward_shot(g, m, case["wavelet"].astype(np.float64), int(sx), int(sz), case["rx"], case["rz"],
                           dtype=np.float64)
        J += 0.5 * float(np.sum((d - dobs[i].astype(np.float64)) ** 2))
    return J


def test_autograd_gradient_matches_finite_differences():
    from pseudoacousticmodeling_gb300.inversion import L2Misfit, Propagate
    case, dobs = _problem()
    e = engine_for(case)
    vp = torch.tensor(case["vp"], dtype=torch.float32, requires_grad=True)
    d = Propagate.apply(vp, e, case["sz"], case["sx"], 0, "f32")
    loss = 0.5 * ((d.double() - torch.from_numpy(dobs).double()) ** 2).sum()
    loss.backward()
    g_auto = vp.grad.numpy().astype(np.float64)

    vp2 = torch.tensor(case["vp"], dtype=torch.float32, requires_grad=True)
    J = L2Misfit.apply(vp2, e, case["sz"], case["sx"], dobs, 40, "f32")
    J.backward()
    assert rel(vp2.grad.numpy(), g_auto) < 1e-6
    assert abs(J.detach().item() - loss.detach().item()) <= 1e-5 * loss.detach().item()

    rng = np.random.default_rng(0)
    g = case["grid"]
    cells = [(int(rng.integers(2, g.nz - 2)), int(rng.integers(2, g.nx - 2))) for _ in range(32)]
    base = case["vp"].astype(np.float64)
    fd = []
    h = 0.25
    for z, x in cells:
        vpp = base.copy(); vpp[z, x] += h
        vpm = base.copy(); vpm[z, x] -= h
        fd.append((_oracle_misfit(case, vpp, dobs) - _oracle_misfit(case, vpm, dobs)) / (2 * h))
    fd = np.array(fd)
    ga = np.array([g_auto[z, x] for z, x in cells])
    err = rel(ga, fd)
    print(f"autograd vs central differences at 32 cells: rel L2 {err:.2e} (|grad| {np.abs(fd).max():.2e})")
    assert err < 1e-2


def test_lbfgs_reduces_misfit():
    from pseudoacousticmodeling_gb300.inversion import fwi
    case, dobs = _problem(seed=13)
    e = engine_for(case)
    inv = fwi(e, case["sz"], case["sx"], dobs, vmin=1400.0, vmax=3200.0, ckpt_interval=60)
    vp = inv.solveFullWaveformInversion(case["vp"], niter=3)
    print("FWI history", inv.history)
    assert np.isfinite(vp).all()
    assert inv.history[-1] < 0.98


def test_multiscale_fwi_per_band_engines():
    """Frequency continuation: one engine per cutoff frequency (its own lag
    and step count), the observed data of each band modelled on the true
    model by an engine of that band, misfit lowered in each band."""
    from pseudoacousticmodeling_gb300 import Config, Engine
    from pseudoacousticmodeling_gb300.inversion import solve_multiscale
    case, _ = _problem(seed=14)
    g = case["grid"]
    true = case["vp"].copy()
    zc = g.nz // 4
    true[zc - 3:zc + 3, g.nx // 2 - 8:g.nx // 2 + 8] += 250.0
    nt_data = g.nt - g.itlag

    def make_engine(fc):
        itlag = int(round(2.0 * np.sqrt(np.pi) / fc / g.dt))
        e = Engine(Config(nz=g.nz, nx=g.nx, n_abc=g.N, dz=g.dz, dx=g.dx, dt=g.dt, nt=itlag + nt_data, itlag=itlag,
                          fcut=fc, approximation="acoustic", boundary="cerjan", max_shots=len(case["sx"])))
        e.set_receivers(case["rz"], case["rx"])
        return e

    def observed(fc):
        e = make_engine(fc)
        e.set_models(true)
        d = e.forward(case["sz"], case["sx"])
        e.close()
        return d

    vp, hist = solve_multiscale(make_engine, case["sz"], case["sx"], observed, [15.0, 30.0], case["vp"], niter=2,
                                vmin=1400.0, vmax=3200.0, ckpt_interval=60)
    print("multiscale FWI histories", hist)
    assert np.isfinite(vp).all()
    assert all(h[-1] < 1.0 for h in hist.values())


def test_lbfgs_on_the_gpu_matches_the_host_loop():
    """The device-resident FWI loop (objective by device modelling and a
    device misfit reduction, L-BFGS vectors as CUDA tensors) against the same
    loop in numpy on the host: same objective and gradient at the start (up to
    the order of the misfit sums) and the same misfit history."""
    from pseudoacousticmodeling_gb300.inversion import fwi
    case, dobs = _problem(seed=13)
    e = engine_for(case)
    gpu = fwi(e, case["sz"], case["sx"], dobs, vmin=1400.0, vmax=3200.0, ckpt_interval=60, device="cuda")
    cpu = fwi(e, case["sz"], case["sx"], dobs, vmin=1400.0, vmax=3200.0, ckpt_interval=60, device="cpu")
    m = 1.0 / np.asarray(case["vp"], np.float64) ** 2
    Xg = gpu.objective_function(gpu._arr(m))
    Xc = cpu.objective_function(m)
    assert abs(Xg - Xc) <= 1e-6 * Xc
    Jg, gg = gpu.calculate_gradient(gpu._arr(m))
    Jc, gc = cpu.calculate_gradient(m)
    assert Jg == Jc and rel(gg.cpu().numpy(), gc) < 1e-12
    vg = gpu.solveFullWaveformInversion(case["vp"], niter=2)
    vc = cpu.solveFullWaveformInversion(case["vp"], niter=2)
    print("FWI history GPU", gpu.history, "host", cpu.history)
    assert np.allclose(gpu.history, cpu.history, rtol=1e-5) and rel(vg, vc) < 1e-5


def test_adjoint_gradient_of_a_given_adjoint_source():
    """pam_adjoint_gradient applies the exact adjoint to the adjoint source
    itself: with the residual d - dobs it is pam_misfit_gradient's gradient
    bit for bit, it scales exactly (2a gives 2 g), and it passes the
    dot-product test <F'(vp) dv, a> = <dv, F'(vp)^T a> against central
    differences of the forward map (FP64 oracle) along a smooth dv."""
    case, dobs = _problem(seed=21)
    e = engine_for(case)
    d = e.forward(case["sz"], case["sx"])
    _, g_ref = e.misfit_gradient(case["sz"], case["sx"], dobs)
    g = e.adjoint_gradient(case["sz"], case["sx"], d - dobs)
    assert np.array_equal(g, g_ref)
    rng = np.random.default_rng(4)
    a = rng.standard_normal(d.shape).astype(np.float32)
    ga = e.adjoint_gradient(case["sz"], case["sx"], a)
    assert np.array_equal(e.adjoint_gradient(case["sz"], case["sx"], 2.0 * a), 2.0 * ga)
    # dot-product test through the FP64 oracle's forward map
    g_ = case["grid"]
    zz, xx = np.meshgrid(np.arange(g_.nz), np.arange(g_.nx), indexing="ij")
    dv = (np.exp(-((zz - g_.nz / 3) ** 2 + (xx - g_.nx / 2) ** 2) / 60.0) * 20.0).astype(np.float64)
    h = 1.0

    def fwd(vp):
        c = dict(case)
        c["vp"] = vp
        m = oracle_models(c)
        m = O.Models(vp=O.expand_model(np.asarray(vp, np.float64), g_.N), A=m.A.astype(np.float64))
        return np.stack([O.forward_shot(g_, m, case["wavelet"].astype(np.float64), int(sx), int(sz), case["rx"],
                                        case["rz"], dtype=np.float64) for sx, sz in zip(case["sx"], case["sz"])])
    vp0 = case["vp"].astype(np.float64)
    jv = (fwd(vp0 + h * dv) - fwd(vp0 - h * dv)) / (2 * h)
    lhs = float(np.sum(jv * a.astype(np.float64)))
    rhs = float(np.sum(dv * ga.astype(np.float64)))
    print(f"adjoint source: <J dv, a> {lhs:.6e}, <dv, J^T a> {rhs:.6e}, rel diff {abs(lhs - rhs) / abs(lhs):.2e}")
    assert abs(lhs - rhs) < 1e-3 * abs(lhs)


def test_autograd_through_a_non_l2_loss():
    """Propagate's backward hands dL/dd to the exact adjoint unchanged, so a
    loss other than the L2 misfit differentiates like the engine's adjoint
    of that dL/dd."""
    from pseudoacousticmodeling_gb300.inversion import Propagate
    case, dobs = _problem(seed=22)
    e = engine_for(case)
    w = torch.from_numpy(np.random.default_rng(6).standard_normal(dobs.shape).astype(np.float32))
    vp = torch.tensor(case["vp"], dtype=torch.float32, requires_grad=True)
    d = Propagate.apply(vp, e, case["sz"], case["sx"], 0, "f32")
    loss = (w * d).sum() + 1e-3 * (d ** 2).sum()
    loss.backward()
    dL = (w + 2e-3 * d.detach()).numpy()
    g = e.adjoint_gradient(case["sz"], case["sx"], dL)
    assert np.isfinite(vp.grad.numpy()).all() and np.abs(g).max() > 0
    assert rel(vp.grad.numpy(), g) < 1e-6
