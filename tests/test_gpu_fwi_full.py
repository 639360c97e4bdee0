"""The acoustic FWI gradient on the full 501 x 1701 grid of the FWI
configuration (10 m cells, 50-cell Cerjan border, band-limited 8 Hz source),
with a truncated time axis so that the checks finish in seconds:

- the checkpointed gradient (plan sized to a budget) equals the
  stored-every-step gradient bitwise;
- the exact gradient against fourth-order central differences of the misfit
  at 32 random cells where the gradient is large;
- the exact gradient against the reference-form gradient of
  cpp/inversion.cu:142-213 (a different discretisation of the same
  derivative, taken with respect to m = 1/vp^2): their cosine;
- the engine's reference-form gradient of one shot against the oracle's
  restatement of cpp/inversion.cu:142-213 at this size, in float64, next to
  the distance of the oracle's own FP32 run from its float64 run.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import rel

pytestmark = pytest.mark.gpu

NT_DATA = 700
SHOTS = 8


@pytest.fixture(scope="module")
def setup():
    from pseudoacousticmodeling_gb300 import Engine, build
    from pseudoacousticmodeling_gb300.workloads import fwi_acoustic
    build.build()
    wl, vtrue, w = fwi_acoustic(shots=SHOTS)
    wl.nt_data = NT_DATA
    w = np.ascontiguousarray(w[:wl.nt])
    e = Engine(wl.config())
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    e.set_models(vtrue)
    dobs = e.forward(wl.sz, wl.sx)
    e.set_models(wl.vp)
    yield wl, vtrue, w, e, dobs
    e.close()


def test_full_grid_checkpointed_gradient_is_exact(setup):
    wl, _, _, e, dobs = setup
    slot = e.field_bytes() * SHOTS
    K, rec = e.plan_checkpoints(wl.nt // 3 * slot)
    assert K > 0 and rec > 0
    a = e.misfit_gradient(wl.sz, wl.sx, dobs, ckpt_interval=0)
    b = e.misfit_gradient(wl.sz, wl.sx, dobs, ckpt_interval=K)
    print(f"full grid, {wl.nt} steps: checkpoint interval {K} ({rec} steps recomputed), misfit {a[0]:.6e}")
    assert a[0] > 0 and a[0] == b[0] and np.array_equal(a[1], b[1])


def test_full_grid_gradient_against_central_differences(setup):
    wl, _, _, e, dobs = setup
    J0, g = e.misfit_gradient(wl.sz, wl.sx, dobs, ckpt_interval=0)
    rng = np.random.default_rng(3)
    # 32 cells among the largest gradients in the illuminated upper half
    upper = np.abs(g[: wl.nz // 2])
    cand = np.argsort(upper.ravel())[-2000:]
    cells = rng.choice(cand, 32, replace=False)
    zs, xs = np.unravel_index(cells, upper.shape)
    fd = np.empty(32)
    h = 5.0                                              # m/s
    for i, (z, x) in enumerate(zip(zs, xs)):
        J = {}
        for k in (1, -1, 2, -2):
            vp = wl.vp.copy()
            vp[z, x] += np.float32(k * h)
            e.set_models(vp)
            d = e.forward(wl.sz, wl.sx)
            r = (d - dobs).astype(np.float64)
            J[k] = 0.5 * float(np.sum(r * r))
        fd[i] = (8.0 * (J[1] - J[-1]) - (J[2] - J[-2])) / (12.0 * h)
    e.set_models(wl.vp)
    an = g[zs, xs].astype(np.float64)
    err = float(np.linalg.norm(an - fd) / np.linalg.norm(fd))
    print(f"full grid: exact gradient vs fourth-order central differences at 32 cells: rel L2 {err:.2e}")
    # the residual is small next to the field a single cell scatters, so the
    # misfit's third derivative in one cell's velocity is large: second-order
    # central differences measured 5.5e-3 at h = 2 m/s and 1.1e-2 at 5 m/s
    # (truncation), the fourth-order stencil removes that term and leaves the
    # FP32 rounding noise of the misfit differences
    assert err < 1e-2


def test_full_grid_exact_and_reference_form_gradients_agree(setup):
    wl, _, _, e, dobs = setup
    _, g_vp = e.misfit_gradient(wl.sz, wl.sx, dobs, ckpt_interval=0)
    e.rtm_reset()
    e.fwi_gradient(wl.sz, wl.sx, dobs, ckpt_interval=0)
    g_ref, _ = e.fwi_result()
    # the reference form is a positive multiple of dJ/dm with respect to
    # m = 1/vp^2 (its adjoint source dobs - dcal and its second time
    # difference of the source field carry one sign each): compare directions
    # with the chain rule dJ/dvp = dJ/dm * (-2 / vp^3)
    vp = wl.vp.astype(np.float64)
    g_ref_vp = g_ref.astype(np.float64) * (-2.0 / vp ** 3)
    # the border folds into the edge cells of the exact gradient only; compare inside
    sl = (slice(5, -5), slice(5, -5))
    a, b = g_vp[sl].ravel().astype(np.float64), g_ref_vp[sl].ravel()
    cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
    print(f"full grid: exact vs reference-form gradient cosine {cos:.5f}")
    assert cos > 0.95


def test_full_grid_reference_form_gradient_matches_oracle(setup):
    wl, _, w, e, dobs = setup
    nt = wl.nt                    # the whole window: reflections make the residual
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=nt, itlag=wl.itlag, fcut=wl.fcut)
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.engine import Config
    e1 = Engine(Config(nz=wl.nz, nx=wl.nx, n_abc=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=nt, itlag=wl.itlag,
                       fcut=wl.fcut, max_shots=1))
    e1.set_wavelet(np.ascontiguousarray(w[:nt]))
    e1.set_receivers(wl.rz, wl.rx)
    e1.set_models(wl.vp)
    d_obs = np.ascontiguousarray(dobs[:1, : nt - wl.itlag])
    e1.rtm_reset()
    mis = e1.fwi_gradient(wl.sz[:1], wl.sx[:1], d_obs, ckpt_interval=97)
    grad, _ = e1.fwi_result()
    e1.close()
    m = O.Models.build(g, wl.vp)
    rg = {}
    for dt in (np.float64, np.float32):
        d = O.forward_shot(g, m, w[:nt], int(wl.sx[0]), int(wl.sz[0]), wl.rx, wl.rz, dtype=dt)
        res = d_obs[0].astype(dt) - d
        rg[dt], _ = O.fwi_gradient_shot(g, m, w[:nt], int(wl.sx[0]), int(wl.sz[0]), wl.rx, wl.rz, res, dtype=dt)
    err = rel(grad, rg[np.float64])
    err32 = rel(grad, rg[np.float32])
    floor = rel(rg[np.float32], rg[np.float64])
    print(f"full grid, one shot, {nt} steps: reference-form gradient vs float64 oracle {err:.2e} "
          f"(FP32 oracle {floor:.2e}), vs FP32 oracle {err32:.2e}")
    # the reference form correlates with the second time difference of the
    # source field, which divides FP32 rounding of P by (omega dt)^2 ~ 4e-5
    # at 8 Hz and dt = 1 ms: any FP32 run of it is a few percent from float64
    # at this size (measured 4.5e-2 for the oracle), mostly the same rounding
    # in both FP32 runs (engine vs FP32 oracle measured 4.2e-3)
    assert mis > 0 and err < 2.0 * floor + 1e-5 and err32 < 1e-2
