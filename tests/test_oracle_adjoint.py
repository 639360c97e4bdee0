"""The exact discrete adjoint of the oracle against finite differences.

misfit_and_exact_gradient transposes the forward scheme of forward_shot
(cpp/Modeling.cu:433-479 with race-free Cerjan damping).  Central differences
of the FP64 misfit with respect to vp at single expanded-grid cells must match
dJ/dvp = dJ/dkappa * 2 vp dt^2.
"""
import numpy as np

from oracle import oracle as O


def _case():
    nz, nx, N = 16, 22, 10
    g = O.Grid(nz=nz, nx=nx, N=N, dz=10.0, dx=10.0, dt=0.001, nt=140, itlag=20, fcut=35.0)
    vp = np.full((nz, nx), 1800.0)
    vp[8:, :] = 2300.0
    m = O.Models.build(g, vp)
    m.vp = m.vp.astype(np.float64)
    m.A = m.A.astype(np.float64)
    true = O.Models.build(g, vp)
    true.vp = true.vp.astype(np.float64).copy()
    true.vp[N + 10:N + 13, N + 9:N + 12] += 150.0
    true.A = m.A
    src = O.ricker_cpp(g.nt, g.dt, g.fcut, 2.0 * np.sqrt(np.pi) / g.fcut, g.dx, g.dz).astype(np.float64)
    sx, sz = N + 6, N + 2
    rx = np.arange(N, N + nx, 2)
    rz = np.full(rx.size, N + 3)
    dobs = O.forward_shot(g, true, src, sx, sz, rx, rz, dtype=np.float64)
    return g, m, src, sx, sz, rx, rz, dobs


def test_exact_gradient_matches_finite_differences():
    g, m, src, sx, sz, rx, rz, dobs = _case()
    J0, gk = O.misfit_and_exact_gradient(g, m, src, sx, sz, rx, rz, dobs, dtype=np.float64)
    assert J0 > 0
    gvp = gk * 2.0 * m.vp * g.dt * g.dt
    cells = [(g.N + 11, g.N + 10), (g.N + 5, g.N + 15), (g.N + 12, g.N + 4), (g.N + 2, g.N + 18),
             (4 + 2, g.N + 8)]      # the last one lies in the Cerjan border
    for z, x in cells:
        h = 0.5
        mp = O.Models(vp=m.vp.copy(), A=m.A)
        mm = O.Models(vp=m.vp.copy(), A=m.A)
        mp.vp[z, x] += h
        mm.vp[z, x] -= h
        Jp = 0.5 * np.sum((O.forward_shot(g, mp, src, sx, sz, rx, rz) - dobs) ** 2)
        Jm = 0.5 * np.sum((O.forward_shot(g, mm, src, sx, sz, rx, rz) - dobs) ** 2)
        fd = (Jp - Jm) / (2 * h)
        assert abs(fd - gvp[z, x]) <= 1e-4 * abs(fd) + 1e-12 * J0, (z, x, fd, gvp[z, x])


def test_exact_adjoint_dot_product():
    """<L dm, dd> = <dm, L^T dd> for the linearised modelling operator, through
    the same routine: the gradient of 0.5 |d(m) - dobs|^2 at dobs = d(m) + eps*dd
    is -eps L^T dd (to first order) while the directional derivative of d is L dm."""
    g, m, src, sx, sz, rx, rz, _ = _case()
    rng = np.random.default_rng(1)
    d0 = O.forward_shot(g, m, src, sx, sz, rx, rz)
    dd = rng.standard_normal(d0.shape)
    eps = 1e-3
    _, gk = O.misfit_and_exact_gradient(g, m, src, sx, sz, rx, rz, d0 + eps * dd, dtype=np.float64)
    LT_dd = -gk / eps                                  # L^T dd with respect to kappa
    dm = np.zeros_like(m.vp)
    dm[4:-4, 4:-4] = rng.standard_normal(dm[4:-4, 4:-4].shape)
    kap = m.vp * m.vp * g.dt * g.dt
    h = 1e-6
    mp = O.Models(vp=np.sqrt((kap + h * dm) / (g.dt * g.dt)), A=m.A)
    mm = O.Models(vp=np.sqrt((kap - h * dm) / (g.dt * g.dt)), A=m.A)
    L_dm = (O.forward_shot(g, mp, src, sx, sz, rx, rz) - O.forward_shot(g, mm, src, sx, sz, rx, rz)) / (2 * h)
    lhs = float(np.sum(L_dm * dd))
    rhs = float(np.sum(dm * LT_dd))
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs))
