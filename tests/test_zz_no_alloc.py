"""pam_misfit_noalloc: the misfit entry point for callers that cannot allocate
device memory where they need the number (a solver loop or serving process
whose device memory was sized once up front).  It must give the same misfit as the gradient entry point on the same
data, call after call, although every call reuses one fixed scratch array in
the library's device image.

This file is collected last on purpose, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from tests.gpu_cases import engine_for, make_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-5   # relative, the bar of the forward parity tests


@pytest.fixture(scope="module")
def lib():
    from pseudoacousticmodeling_gb300 import _lib, build
    build.build()
    return _lib.load()


def _noalloc(lib, dcal, dobs):
    out = ctypes.c_double(-1.0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.pam_misfit_noalloc(ctypes.c_void_p(dcal.data_ptr()), ctypes.c_void_p(dobs.data_ptr()),
                                dcal.numel(), ctypes.byref(out), ctypes.c_void_p(stream))
    assert rc == 0
    return out.value


def test_noalloc_misfit_matches_gradient_entry_point(lib):
    case = make_case("acoustic", "cerjan", nt=300, nshots=3, seed=21)
    e = engine_for(case)
    dcal = e.forward(case["sz"], case["sx"])
    rng = np.random.default_rng(5)
    dobs_a = (dcal + 1e-3 * np.abs(dcal).max() * rng.standard_normal(dcal.shape)).astype(np.float32)
    dobs_b = (0.9 * dcal[:1]).astype(np.float32)

    # the existing entry point on the same data (it models dcal itself)
    J_a, _ = e.misfit_gradient(case["sz"], case["sx"], dobs_a)
    J_b, _ = e.misfit_gradient(case["sz"][:1], case["sx"][:1], dobs_b)

    d_dcal = torch.from_numpy(dcal).cuda()
    first = _noalloc(lib, d_dcal, torch.from_numpy(dobs_a).cuda())
    # second call: a smaller input; what the first call left in the scratch
    # array must not leak into it
    second = _noalloc(lib, d_dcal[:1].contiguous(), torch.from_numpy(dobs_b).cuda())
    print(f"no-alloc misfit {first:.6e} / {second:.6e}; gradient entry point {J_a:.6e} / {J_b:.6e}")
    assert abs(first - J_a) <= TOL * J_a
    assert abs(second - J_b) <= TOL * J_b
    # and the first input again, after the smaller one
    again = _noalloc(lib, d_dcal, torch.from_numpy(dobs_a).cuda())
    assert abs(again - J_a) <= TOL * J_a


def test_noalloc_rejects_oversized_input(lib):
    too_many = 134217728 + 1
    x = torch.zeros(4, device="cuda")
    out = ctypes.c_double(0.0)
    rc = lib.pam_misfit_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), too_many,
                                ctypes.byref(out), None)
    assert rc == -1   # PAM_E_ARG, before any launch
