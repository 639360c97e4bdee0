"""RTM imaging, the reference FWI gradient and the exact gradient on the GPU,
against the CPU oracle.

Bars (relative L2): images within 1e-4 of the FP32 oracle (they accumulate
products of two FP32 wavefields over every step) and gradients within 1e-3
(the FWI bar; against the FP64 oracle for the exact gradient).  Checkpointed
reconstruction with FP32 checkpoints is bitwise equal to storing every step.
Compressed checkpoints perturb the rebuilt source field at every segment
start; the error they cause is measured and bounded here: images within 1e-2
of FP32 for both formats, exact gradients within 5e-3 (FP16 with a
per-snapshot scale, 11-bit mantissa) and 5e-2 (BF16, 8-bit mantissa) of FP64.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import engine_for, make_case, oracle_models, rel

pytestmark = pytest.mark.gpu

TOL_IMG = 1e-4
TOL_GRAD = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


def _observed(case, bump=300.0, dtype=np.float32):
    """Data of a model with a shallow box anomaly (reached by the recorded
    wavefield within the run), modelled by the FP32 oracle."""
    g = case["grid"]
    vp = case["vp"].copy()
    zc = g.nz // 5
    vp[zc - 3:zc + 3, g.nx // 2 - 8:g.nx // 2 + 8] += bump
    c2 = dict(case)
    c2["vp"] = vp
    m = oracle_models(c2)
    return np.stack([O.forward_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dtype=dtype)
                     for sx, sz in zip(case["sx"], case["sz"])]).astype(np.float32)


def _oracle_rtm(case, dobs, dtype):
    g = case["grid"]
    m = oracle_models(case)
    img = np.zeros((g.nz, g.nx))
    ilum = np.zeros((g.nz, g.nx))
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        a, b = O.rtm_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dobs[i], dtype=dtype)
        img += a
        ilum += b
    return img, ilum


@pytest.mark.parametrize("approx,abc,sd_off", [("acoustic", "cerjan", False), ("acoustic", "CPML", False),
                                               ("VTI", "cerjan", True), ("TTI", "cerjan", True),
                                               ("VTI", "cerjan", False), ("TTI", "cerjan", False)])
def test_rtm_matches_oracle(approx, abc, sd_off):
    """Images and illumination against the FP32 oracle; the anisotropic cases
    with the pseudo-acoustic Sd term removed (delta = epsilon) and active."""
    case = make_case(approx, abc, nt=220, sd_off=sd_off)
    dobs = _observed(case)
    e = engine_for(case)
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    img, ilum = e.rtm_result(norm="none")
    r_img, r_ilum = _oracle_rtm(case, dobs, np.float32)
    e_img, e_il = rel(img, r_img), rel(ilum, r_ilum)
    print(f"RTM {approx}/{abc} Sd {'off' if sd_off else 'on'}: image {e_img:.2e}, illumination {e_il:.2e}")
    assert np.abs(r_img).max() > 0
    assert e_img < TOL_IMG and e_il < TOL_IMG
    # the C++ normalisation (cpp/Migration.cu:470-484)
    norm, _ = e.rtm_result(norm="cpp")
    assert rel(norm, O.normalize_image_cpp(r_img, r_ilum)) < 10 * TOL_IMG


@pytest.mark.parametrize("abc", ["cerjan", "CPML"])
def test_checkpointed_rtm_is_exact(abc):
    case = make_case("acoustic", abc, nt=230, seed=4)
    dobs = _observed(case)
    e = engine_for(case)
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    full, il_full = e.rtm_result(norm="none")
    for K in (17, 50):
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=K, store="f32")
        img, il = e.rtm_result(norm="none")
        assert np.array_equal(img, full) and np.array_equal(il, il_full)
    for store in ("bf16", "f16"):
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=23, store=store)
        img, _ = e.rtm_result(norm="none")
        err = rel(img, full)
        print(f"{abc} {store} checkpoints: image rel L2 vs FP32 {err:.2e}")
        assert err < 1e-2


def test_fwi_reference_gradient_matches_oracle():
    case = make_case("acoustic", "cerjan", nt=330, seed=6)
    dobs = _observed(case)
    e = engine_for(case)
    mis = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=31)
    grad, ilum = e.fwi_result()
    g = case["grid"]
    m = oracle_models(case)
    rg = np.zeros((g.nz, g.nx))
    ri = np.zeros((g.nz, g.nx))
    rmis = 0.0
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        d = O.forward_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dtype=np.float32)
        res = dobs[i] - d
        rmis += 0.5 * float(np.sum(res.astype(np.float64) ** 2))
        a, b = O.fwi_gradient_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], res,
                                   dtype=np.float32)
        rg += a
        ri += b
    print(f"FWI reference gradient: {rel(grad, rg):.2e}, illumination {rel(ilum, ri):.2e}, "
          f"misfit {abs(mis - rmis) / rmis:.2e}")
    assert rmis > 1e-6 * 0.5 * float(np.sum(dobs.astype(np.float64) ** 2))   # the anomaly is in the data
    assert rel(grad, rg) < TOL_GRAD and rel(ilum, ri) < TOL_IMG
    assert abs(mis - rmis) <= 1e-3 * rmis


GRAD_BOUND = {"f32": TOL_GRAD, "f16": 5e-3, "bf16": 5e-2}


@pytest.mark.parametrize("K,store", [(0, "f32"), (29, "f32"), (29, "f16"), (29, "bf16")])
def test_exact_gradient_matches_fp64_oracle(K, store):
    case = make_case("acoustic", "cerjan", nt=330, seed=8)
    dobs = _observed(case)
    e = engine_for(case)
    mis, gvp = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=K, store=store)
    g = case["grid"]
    m = oracle_models(case)
    m64 = O.Models(vp=m.vp.astype(np.float64), A=m.A.astype(np.float64))
    gk = np.zeros((g.nz_a, g.nx_a))
    J = 0.0
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        j, k = O.misfit_and_exact_gradient(g, m64, case["wavelet"].astype(np.float64), int(sx), int(sz),
                                           case["rx"], case["rz"], dobs[i].astype(np.float64))
        J += j
        gk += k
    # chain rule kappa = vp^2 dt^2 and the transpose of the edge padding
    N = g.N
    gv = gk * 2.0 * m64.vp * g.dt * g.dt
    ref = np.zeros((g.nz, g.nx))
    for z in range(g.nz_a):
        zi = min(max(z - N, 0), g.nz - 1)
        np.add.at(ref[zi], np.clip(np.arange(g.nx_a) - N, 0, g.nx - 1), gv[z])
    err = rel(gvp, ref)
    print(f"exact gradient K={K} {store}: rel L2 vs FP64 {err:.2e}, misfit {abs(mis - J) / J:.2e}")
    assert err < GRAD_BOUND[store]
    assert abs(mis - J) <= 1e-3 * J


@pytest.mark.parametrize("approx", ["VTI", "TTI"])
def test_multiparameter_reference_gradient_matches_oracle(approx):
    """The reference-form FWI gradient of an anisotropic model with the
    multiparameter terms (src/utils.py:1309-1463) against the oracle (FP32
    fields, float64 per-cell formula as the reference's numba code)."""
    case = make_case(approx, "cerjan", nt=300, seed=9, sd_off=True)
    dobs = _observed(case)
    e = engine_for(case)
    e.set_multiparameter(True)
    mis = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=37)
    gvp, ilum = e.fwi_result()
    ge, gd, gt = e.fwi_multiparameter_result()
    g = case["grid"]
    m = oracle_models(case)
    r = [np.zeros((g.nz, g.nx)) for _ in range(5)]
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        d = O.forward_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dtype=np.float32)
        res = dobs[i] - d
        out = O.multiparameter_fwi_gradient_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"],
                                                 res, dtype=np.float32)
        for k in range(5):
            if out[k] is not None:
                r[k] += out[k]
    errs = {"vp": rel(gvp, r[0]), "eps": rel(ge, r[1]), "delta": rel(gd, r[2]), "ilum": rel(ilum, r[4])}
    if approx == "TTI":
        errs["theta"] = rel(gt, r[3])
    print(f"multiparameter FWI {approx}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert np.abs(r[1]).max() > 0 and mis > 0
    assert errs["vp"] < TOL_GRAD and errs["ilum"] < TOL_IMG
    assert errs["eps"] < TOL_GRAD and errs["delta"] < TOL_GRAD and errs.get("theta", 0.0) < TOL_GRAD


def test_pinned_observed_data_give_identical_results():
    """Observed data in pinned memory upload on a copy stream while the
    forward sweep runs; misfits, gradients and images must equal those of
    pageable data bitwise, for every source-field strategy that reads them at a
    different point (checkpoints, every step stored, boundary saving)."""
    torch = pytest.importorskip("torch")
    case = make_case("acoustic", "cerjan", nt=300, seed=10)
    dobs = _observed(case)
    pinned = torch.empty(dobs.shape, dtype=torch.float32).pin_memory().numpy()
    pinned[:] = dobs
    e = engine_for(case)
    for K in (31, 0):
        a = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=K)
        b = e.misfit_gradient(case["sz"], case["sx"], pinned, ckpt_interval=K)
        assert a[0] == b[0] and np.array_equal(a[1], b[1])
    for K in (0, -1):     # every step stored; boundary saving
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=K)
        img_a, _ = e.rtm_result(norm="none")
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], pinned, ckpt_interval=K)
        img_b, _ = e.rtm_result(norm="none")
        assert np.array_equal(img_a, img_b) and np.abs(img_a).max() > 0
    e.rtm_reset()      # the reference-form gradient accumulates until reset
    ma = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=-1)
    ga, _ = e.fwi_result()
    e.rtm_reset()
    mb = e.fwi_gradient(case["sz"], case["sx"], pinned, ckpt_interval=-1)
    gb, _ = e.fwi_result()
    assert ma == mb and np.array_equal(ga, gb)


def test_gpu_mute_matches_the_host_mute():
    """pam_set_mute arms the mute of Migration::Mute (cpp/Migration.cu:86-115)
    for the next migration call, applied on the GPU after the upload: the
    image must equal, bitwise, that of the same data muted on the host by the
    float32 restatement, with shared and per-shot receiver coordinates and with
    pageable and pinned data; the mute is used up by one call, and a call with
    another shot count is refused."""
    torch = pytest.importorskip("torch")
    from pseudoacousticmodeling_gb300 import PamError, preprocess
    case = make_case("acoustic", "cerjan", nt=300, seed=11)
    g = case["grid"]
    dobs = _observed(case)
    # metres, off the grid so that t1 falls between samples
    shot_x = ((case["sx"] - g.N) * g.dx + 3.3).astype(np.float32)
    shot_z = ((case["sz"] - g.N) * g.dz + 1.1).astype(np.float32)
    rec_x = ((case["rx"] - g.N) * g.dx + 1.7).astype(np.float32)
    rec_z = ((case["rz"] - g.N) * g.dz + 0.4).astype(np.float32)
    v0, shift, window = 1500.0, 0.02, 0.035
    e = engine_for(case)

    def image(d, **mute):
        e.rtm_reset()
        if mute:
            e.set_mute(shot_x, shot_z, mute["rx"], mute["rz"], v0, shift, window)
        e.rtm(case["sz"], case["sx"], d, ckpt_interval=0)
        return e.rtm_result(norm="none")[0]

    ns = len(case["sx"])
    rx2 = np.stack([rec_x + 2.5 * i for i in range(ns)]).astype(np.float32)
    rz2 = np.stack([rec_z] * ns).astype(np.float32)
    for rx, rz in ((rec_x, rec_z), (rx2, rz2)):
        host = np.stack([preprocess.mute(dobs[i], rx if rx.ndim == 1 else rx[i], rz if rz.ndim == 1 else rz[i],
                                         shot_x[i], shot_z[i], g.dt, v0, shift, window) for i in range(ns)])
        assert (host == 0).any() and not np.array_equal(host, dobs)
        ref = image(host)
        assert np.array_equal(image(dobs, rx=rx, rz=rz), ref)
        pinned = torch.empty(dobs.shape, dtype=torch.float32).pin_memory().numpy()
        pinned[:] = dobs
        assert np.array_equal(image(pinned, rx=rx, rz=rz), ref)
    raw = image(dobs)                                   # the mute was used up
    assert not np.array_equal(raw, ref)
    e.set_mute(shot_x[:2], shot_z[:2], rec_x, rec_z, v0, shift, window)
    with pytest.raises(PamError, match="armed for 2 shots"):
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    e.clear_mute()


def test_checkpoint_planner_and_kept_last_segment():
    """pam_plan_checkpoints picks the interval with the fewest recomputed
    steps whose buffers fit the budget; the forward sweep keeps the last
    segment in the segment buffer, so any interval gives the misfit and exact
    gradient of storing every step, bitwise."""
    from pseudoacousticmodeling_gb300 import PamError
    case = make_case("acoustic", "cerjan", nt=230, seed=12)
    dobs = _observed(case)
    e = engine_for(case)
    nt = case["grid"].nt
    slot = e.field_bytes() * len(case["sx"])
    assert e.plan_checkpoints(10 ** 15) == (0, 0)          # everything fits: store every step
    for budget_slots in (nt // 2 + 5, nt // 3 + 8, 50):
        budget = budget_slots * slot
        K, rec = e.plan_checkpoints(budget)
        nseg = -(-nt // K)
        assert K > 0 and (K + 2) * slot + (nseg - 1) * 2 * slot <= budget
        assert rec == (nseg - 1) * K
        # one segment fewer would not fit
        Kf = -(-nt // (nseg - 1))
        assert nseg == 2 or (Kf + 2) * slot + (-(-nt // Kf) - 1) * 2 * slot > budget
    with pytest.raises(PamError):
        e.plan_checkpoints(3 * slot)
    ref = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=0)
    for K in (e.plan_checkpoints((nt // 2 + 5) * slot)[0], 57, 115):
        got = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=K)
        assert got[0] == ref[0] and np.array_equal(got[1], ref[1]), K
