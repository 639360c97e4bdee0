"""Known-answer tests without a GPU:
- the 8th-order coefficients as exact fractions and as the float literals that
  the kernels and the reference use;
- the oracle's Laplacian on fields whose derivatives are known exactly;
- the engine-free dispersion / stability check (cpp/Modeling.cu:184-327) at
  limits computed by hand."""
import ctypes
from fractions import Fraction as F

import numpy as np
import pytest

from oracle import oracle as O

# second derivative C_k (k = 0..4), first derivative A_k (k = 1..4)
C = [F(-1435, 504), F(8, 5), F(-1, 5), F(8, 315), F(-1, 560)]
A = [F(4, 5), F(-1, 5), F(4, 105), F(-1, 280)]
# the float literals of cpp/Modeling.cu:500-504, 560-563, also used by the kernels
C_LIT = [-2.847222222222, 1.6, -0.2, 0.02539682539, -0.00178571428]
A_LIT = [0.8, -0.2, 0.03809523809, -0.00357142857]


def test_coefficients_are_eighth_order():
    # sum_k C_k (k^m + (-k)^m) reproduces d2/dx2 of x^m at 0 for m <= 9
    for m in range(0, 10):
        s = C[0] * (1 if m == 0 else 0) + sum(C[k] * (k ** m + (-k) ** m) for k in range(1, 5))
        assert s == (2 if m == 2 else 0), m
    # sum_k A_k (k^m - (-k)^m) reproduces d/dx of x^m at 0 for m <= 8
    for m in range(0, 9):
        s = sum(A[k - 1] * (k ** m - (-k) ** m) for k in range(1, 5))
        assert s == (1 if m == 1 else 0), m


def test_float_literals_round_the_fractions():
    for lit, frac in zip(C_LIT + A_LIT, C + A):
        assert np.float32(lit) == np.float32(float(frac))


def test_oracle_laplacian_known_answers():
    nz, nx, dz, dx = 24, 30, 7.0, 5.0
    z = np.arange(nz, dtype=np.float64)[:, None] * dz
    x = np.arange(nx, dtype=np.float64)[None, :] * dx
    const = np.full((nz, nx), 3.5)
    assert np.abs(O._lap(const, dz, dx, np.float64)).max() < 1e-9
    quad = 2.0 + 0.3 * x - 0.7 * z + 0.05 * x * x + 0.02 * z * z + 0.01 * x * z
    np.testing.assert_allclose(O._lap(quad, dz, dx, np.float64), 0.1 + 0.04, rtol=1e-9)
    # exact for polynomials up to degree 9 in each direction: d2/dx2 x^9 = 72 x^7
    xs = (x - x.mean()) / 40.0
    zs = (z - z.mean()) / 40.0
    poly = xs ** 9 + zs ** 8 + np.zeros((nz, nx))
    ref = 72.0 * xs ** 7 / 40.0 ** 2 + 56.0 * zs ** 6 / 40.0 ** 2
    np.testing.assert_allclose(O._lap(poly, dz, dx, np.float64), ref[4:-4, 4:-4], rtol=1e-7, atol=1e-12)


@pytest.fixture(scope="module")
def lib():
    from pseudoacousticmodeling_gb300 import _lib, build
    build.build()
    return _lib.load()


def _limits(lib, approx, vp, eps=None, delta=None, theta=None, dx=10.0, dz=10.0, dt=1e-4, fcut=30.0):
    nz, nx = vp.shape
    p = lambda a: None if a is None else np.ascontiguousarray(a, np.float32).ctypes.data_as(ctypes.c_void_p)
    keep = [np.ascontiguousarray(a, np.float32) if a is not None else None for a in (vp, eps, delta, theta)]
    dt_lim, dx_lim = ctypes.c_float(), ctypes.c_float()
    rc = lib.pam_stability_limits(approx, nz, nx, *[p(a) for a in keep], dx, dz, dt, fcut, ctypes.byref(dt_lim),
                                  ctypes.byref(dx_lim))
    return rc, dt_lim.value, dx_lim.value


def test_stability_limits_known_values(lib):
    ACOUSTIC, VTI, TTI = 0, 1, 2
    vp = np.full((6, 9), 2500.0, np.float32)
    vp[0, 0], vp[5, 8] = 1500.0, 4000.0
    # acoustic: shortest wavelength vmin / fcut over 4.28 cells; dt <= dx_lim / (4 vmax)
    rc, dt_lim, dx_lim = _limits(lib, ACOUSTIC, vp)
    assert dx_lim == pytest.approx(1500.0 / 30.0 / 4.28, rel=1e-6)
    assert dt_lim == pytest.approx(dx_lim / (4.0 * 4000.0), rel=1e-6)
    assert rc == 1
    assert _limits(lib, ACOUSTIC, vp, dx=12.0)[0] == 0           # too coarse for 30 Hz
    assert _limits(lib, ACOUSTIC, vp, dt=1e-3)[0] == 0           # too long a step
    # VTI with eps = delta = 0: isotropic phase velocity, the leapfrog limit
    # sqrt(2) / (sqrt(sum_m c_m (1 - (-1)^m)) vmax sqrt(1/dx^2 + 1/dz^2))
    z = np.zeros_like(vp)
    rc, dt_v, dx_v = _limits(lib, VTI, vp, z, z)
    soma = 2.0 * (8.0 / 5.0 + 8.0 / 315.0)
    assert dt_v == pytest.approx(np.sqrt(2.0) / (np.sqrt(soma) * 4000.0 * np.sqrt(2.0 / 100.0)), rel=1e-5)
    assert dx_v == pytest.approx(dx_lim, rel=1e-5)
    # epsilon = delta > 0 speeds up every direction but the vertical one: the
    # slowest phase velocity (hence dx_lim) stays, the time-step limit shrinks
    e = np.full_like(vp, 0.2)
    _, dt_e, dx_e = _limits(lib, VTI, vp, e, e)
    assert dx_e == pytest.approx(dx_lim, rel=1e-5) and dt_e < dt_v
    # TTI over 180 degrees of propagation angle: a uniform tilt changes nothing
    _, dt_t, dx_t = _limits(lib, TTI, vp, e, e, np.full_like(vp, 35.0))
    assert dt_t == pytest.approx(dt_e, rel=1e-6) and dx_t == pytest.approx(dx_e, rel=1e-3)
    # invalid arguments
    assert _limits(lib, VTI, vp)[0] == -1                        # eps/delta missing
    assert _limits(lib, TTI, vp, e, e)[0] == -1                  # theta missing
    assert _limits(lib, 7, vp)[0] == -1
