"""This engine's migration against the reference's own migration kernels.

cpp/Modeling.cu and cpp/Migration.cu are compiled unmodified into cubins
(oracle/build.py) and run in the reference's on-the-fly migration loop
(cpp/Migration.cu:359-397, restated on the CUDA driver API in
oracle/ref_harness.cpp: ref_rtm): the forward kernels with the source field
saved after every update, then per backward step injectAdjointSource, the
acoustic adjoint kernel or the anisotropic products and update kernels with
their imaging sums, and normalizeImage at the end.  That loop copies each
saved field on a second stream while the next step runs; the harness orders
the copy after the update instead (the field the reference means to save).

Like the forward kernels, the reference's adjoint kernels damp U in place
while neighbouring threads read it, inside the Cerjan border only.  Images
and illumination are sums over the interior, which that race reaches only
through the fields it perturbs: measured, the engine sits 0.4-1.1e-6 from the
reference kernels in relative L2, as close as the race-free oracle does, so
image, illumination and the C++-normalised image are held to 1e-5, the
forward path's bar, on small grids and on the full batched-VTI grid; the
reference's run-to-run spread and the race-free oracle's distance from it are
printed beside the engine's.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import engine_for, make_case, oracle_models, rel

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as R
    if R.cubin_path() is None or R.migration_cubin_path() is None:
        pytest.skip("the reference cubins were not built: the reference sources were absent where the build ran "
                    "(oracle/build.py reads them from PAM_REFERENCE_SRC)")
    from pseudoacousticmodeling_gb300 import build
    build.build()
    return R


def _observed(case, bump=300.0):
    """Data of the case's model with a shallow box anomaly, modelled by the
    FP32 oracle (the same observed data for both migrations)."""
    g = case["grid"]
    vp = case["vp"].copy()
    zc = g.nz // 5
    vp[zc - 3:zc + 3, g.nx // 2 - 8:g.nx // 2 + 8] += bump
    c2 = dict(case)
    c2["vp"] = vp
    m = oracle_models(c2)
    return np.stack([O.forward_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"],
                                    dtype=np.float32)
                     for sx, sz in zip(case["sx"], case["sz"])]).astype(np.float32)


def _oracle_rtm(case, dobs):
    g = case["grid"]
    m = oracle_models(case)
    img = np.zeros((g.nz, g.nx))
    ilum = np.zeros((g.nz, g.nx))
    for i, (sx, sz) in enumerate(zip(case["sx"], case["sz"])):
        a, b = O.rtm_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dobs[i], dtype=np.float32)
        img += a
        ilum += b
    return img, ilum


@pytest.mark.parametrize("approx,sd_off", [("acoustic", False), ("VTI", False), ("TTI", False), ("VTI", True)])
def test_engine_migration_against_reference_migration_kernels(ref, approx, sd_off):
    case = make_case(approx, "cerjan", nt=220, sd_off=sd_off)
    g = case["grid"]
    dobs = _observed(case)
    m = oracle_models(case)
    args = (g, m, case["wavelet"], case["sx"], case["sz"], case["rx"], case["rz"], dobs)
    r_img, r_ilum, _ = ref.rtm(*args, normalize=False)
    r2_img, _, _ = ref.rtm(*args, normalize=False)
    r_norm, _, _ = ref.rtm(*args, normalize=True)
    assert np.abs(r_img).max() > 0 and np.isfinite(r_img).all()

    e = engine_for(case)
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    img, ilum = e.rtm_result(norm="none")
    norm, _ = e.rtm_result(norm="cpp")
    e.close()
    o_img, _ = _oracle_rtm(case, dobs)

    e_img, e_il, e_norm = rel(img, r_img), rel(ilum, r_ilum), rel(norm, r_norm)
    print(f"\nmigration {approx} Sd {'off' if sd_off else 'on'}: engine vs reference kernels image {e_img:.2e}, "
          f"illumination {e_il:.2e}, C++-normalised {e_norm:.2e} (reference run-to-run {rel(r2_img, r_img):.2e}, "
          f"race-free oracle vs reference {rel(o_img, r_img):.2e})")
    assert e_img < TOL and e_il < TOL and e_norm < TOL


def test_full_grid_vti_migration_against_reference_kernels(ref):
    """The batched-VTI grid (801 x 2001 at 10 m + 50-cell Cerjan border), Sd
    active, 800 time steps, one shot: the engine's migration against the
    reference's on-the-fly migration kernels (which store all 800 source
    fields, 6 GB).  Observed data: the engine's modelling of the model with a
    box anomaly inside the depth the run reaches."""
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.engine import Config
    from pseudoacousticmodeling_gb300.workloads import batched_vti
    wl = batched_vti(shots=1)
    nt, itlag = 800, 40
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=nt, itlag=itlag, fcut=wl.fcut,
               approx="VTI", abc="cerjan")
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta, wl.theta)
    w = O.ricker_cpp(nt, g.dt, g.fcut, np.float32(2.0 * np.sqrt(np.pi) / g.fcut), g.dx, g.dz)
    e = Engine(Config(nz=wl.nz, nx=wl.nx, n_abc=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=nt, itlag=itlag,
                      fcut=wl.fcut, approximation="VTI", boundary="cerjan", max_shots=1))
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    sz, sx = wl.sz[:1], wl.sx[:1]
    vp_b = wl.vp.copy()
    vp_b[40:50, wl.nx // 2 - 30:wl.nx // 2 + 30] += 400.0
    e.set_models(vp_b, wl.eps, wl.delta)
    dobs = e.forward(sz, sx)
    e.set_models(wl.vp, wl.eps, wl.delta)
    e.rtm(sz, sx, dobs, ckpt_interval=0)
    img, ilum = e.rtm_result(norm="none")
    norm, _ = e.rtm_result(norm="cpp")
    e.close()
    args = (g, m, w, sx, sz, wl.rx, wl.rz, dobs)
    r_img, r_ilum, ms = ref.rtm(*args, normalize=False)
    r2_img, _, _ = ref.rtm(*args, normalize=False)
    r_norm, _, _ = ref.rtm(*args, normalize=True)
    assert np.abs(r_img).max() > 0 and np.isfinite(r_img).all()
    e_img, e_il, e_norm = rel(img, r_img), rel(ilum, r_ilum), rel(norm, r_norm)
    print(f"\nmigration VTI 901x2101x800: engine vs reference kernels image {e_img:.2e}, illumination {e_il:.2e}, "
          f"C++-normalised {e_norm:.2e} (reference run-to-run {rel(r2_img, r_img):.2e}; reference kernels "
          f"{ms:.1f} ms per shot)")
    assert e_img < TOL and e_il < TOL and e_norm < TOL
