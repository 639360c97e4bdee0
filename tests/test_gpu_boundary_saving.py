"""Boundary saving (src/Migration.py:288-298, 714-834) on the GPU.

The source field is rebuilt backwards in time from the last two forward
states, writing the saved four-cell band of the physical region back after
every reverse step.  Inside the physical region this is exact up to the
rounding of the reversed recursion, so migration images and the reference
FWI gradient must match the store-every-step results (which the oracle pins)
within 1e-4 and 1e-3.  Compressed bands (BF16 / FP16, one scale per 256 cells)
are measured against the FP32 bands.
"""
import numpy as np
import pytest

from tests.gpu_cases import engine_for, make_case, rel
from tests.test_gpu_adjoint import _observed

pytestmark = pytest.mark.gpu

SB = -1   # PAM_BOUNDARY_SAVING


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


@pytest.mark.parametrize("approx,abc", [("acoustic", "cerjan"), ("acoustic", "CPML"), ("VTI", "cerjan"),
                                        ("TTI", "cerjan")])
def test_boundary_saving_rtm_matches_stored_source_field(approx, abc):
    case = make_case(approx, abc, nt=260, seed=12, sd_off=(approx != "acoustic"))
    dobs = _observed(case)
    e = engine_for(case)
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    full, il_full = e.rtm_result(norm="none")
    e.rtm_reset()
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=SB, store="f32")
    img, il = e.rtm_result(norm="none")
    err_img, err_il = rel(img, full), rel(il, il_full)
    errs = {}
    for store in ("f16", "bf16"):
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=SB, store=store)
        errs[store] = rel(e.rtm_result(norm="none")[0], full)
    print(f"boundary saving RTM {approx}/{abc}: image vs stored field {err_img:.2e}, illumination {err_il:.2e}; "
          f"FP16 bands {errs['f16']:.2e}, BF16 bands {errs['bf16']:.2e}")
    assert np.isfinite(img).all() and np.abs(full).max() > 0
    assert err_img < 1e-4 and err_il < 1e-4
    assert errs["f16"] < 1e-2 and errs["bf16"] < 5e-2


def test_boundary_saving_reference_gradient():
    case = make_case("acoustic", "cerjan", nt=330, seed=6)
    dobs = _observed(case)
    e = engine_for(case)
    mis_ck = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=31)
    g_ck, il_ck = e.fwi_result()
    e2 = engine_for(case)
    mis_sb = e2.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=SB)
    g_sb, il_sb = e2.fwi_result()
    print(f"boundary saving FWI reference gradient: {rel(g_sb, g_ck):.2e}, illumination {rel(il_sb, il_ck):.2e}")
    assert mis_sb == mis_ck
    assert rel(g_sb, g_ck) < 1e-3 and rel(il_sb, il_ck) < 1e-4


def test_boundary_saving_refuses_the_exact_gradient():
    from pseudoacousticmodeling_gb300 import PamError
    case = make_case("acoustic", "cerjan", nt=120, seed=6)
    e = engine_for(case)
    with pytest.raises(PamError, match="boundary saving"):
        e.misfit_gradient(case["sz"], case["sx"], np.zeros((3, case["grid"].nt_data, case["rx"].size), np.float32),
                          ckpt_interval=SB)


RBC = -2  # PAM_RANDOM_BOUNDARY


def _cosine(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))


@pytest.mark.parametrize("approx,abc", [("acoustic", "cerjan"), ("acoustic", "CPML"), ("VTI", "cerjan")])
def test_random_boundary_rtm(approx, abc):
    """The source field runs undamped through a random border and is rebuilt by
    running backwards: reproducible for a seed, and the image differs from the
    stored-field one only by the energy the border scatters back."""
    case = make_case(approx, abc, nt=260, seed=12, sd_off=(approx != "acoustic"))
    dobs = _observed(case)
    e = engine_for(case)
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=0)
    full, il_full = e.rtm_result(norm="none")
    e.set_random_boundary(dvel=600.0, ratio=60.0, seed=3)
    e.rtm_reset()
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=RBC)
    img, il = e.rtm_result(norm="none")
    e.rtm_reset()
    e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=RBC)
    img2, _ = e.rtm_result(norm="none")
    c_img, c_il = _cosine(img, full), _cosine(il, il_full)
    print(f"random boundary RTM {approx}/{abc}: image cosine vs stored field {c_img:.4f}, illumination {c_il:.4f}, "
          f"rel L2 {rel(img, full):.2e}")
    assert np.isfinite(img).all()
    assert np.array_equal(img, img2)
    assert c_img > 0.9 and c_il > 0.9


def test_random_boundary_reference_gradient_and_refusals():
    from pseudoacousticmodeling_gb300 import PamError
    case = make_case("acoustic", "cerjan", nt=330, seed=6)
    dobs = _observed(case)
    e = engine_for(case)
    mis_ck = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=31)
    g_ck, _ = e.fwi_result()
    e2 = engine_for(case)
    e2.set_random_boundary(dvel=600.0, ratio=60.0, seed=1)
    mis_rbc = e2.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=RBC)
    g_rbc, _ = e2.fwi_result()
    c = _cosine(g_rbc, g_ck)
    print(f"random boundary FWI reference gradient: cosine vs checkpoints {c:.4f}")
    assert mis_rbc == mis_ck          # the modelled data come from the absorbing scheme
    assert np.isfinite(g_rbc).all() and c > 0.8
    with pytest.raises(PamError, match="random boundary"):
        e2.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=RBC)
