"""Pin the CPU oracle to the reference.

The fixtures in tests/golden/golden_small.npz are outputs of the reference's
own Python CPU kernels (src/utils.py, src/Modeling2D.py) evaluated in
float64; tests/golden/make_golden.py regenerates them.  The FP64 oracle must
reproduce them to round-off; the FP32 oracle (the reference C++ term order)
to single-precision accuracy.
"""
import numpy as np
import pytest

from oracle import oracle as O


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _grid(G, approx, abc="cerjan"):
    nz, nx, N = int(G["k_nz"]), int(G["k_nx"]), int(G["k_N"])
    return O.Grid(nz=nz - 2 * N, nx=nx - 2 * N, N=N, dz=float(G["k_dz"]), dx=float(G["k_dx"]),
                  dt=float(G["k_dt"]), nt=1, itlag=0, fcut=float(G["k_fcut"]), approx=approx, abc=abc)


def _models(G, g, dtype):
    m = O.Models(vp=G["k_vp"].astype(dtype), eps=G["k_eps"].astype(dtype),
                 delta=G["k_delta"].astype(dtype), theta=G["k_theta"].astype(dtype))
    return m


@pytest.mark.parametrize("approx,key", [("acoustic", "k_acoustic"), ("VTI", "k_vti"), ("TTI", "k_tti")])
@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-12), (np.float32, 2e-6)])
def test_single_step(golden, approx, key, dtype, tol):
    G = golden
    g = _grid(G, approx)
    m = _models(G, g, dtype)
    Uf = G["k_Uf"].astype(dtype).copy()
    Uc = G["k_Uc"].astype(dtype).copy()
    O.step(g, m, Uf, Uc, dtype=dtype)   # no boundary: A and CPML absent
    assert rel(Uf, G[key]) < tol


def test_cerjan_vector_and_damping(golden):
    G = golden
    A64 = G["k_cerjanA"]
    A32 = O.cerjan_vector(int(G["k_N"]))
    assert rel(A32, A64) < 1e-6
    g = _grid(G, "acoustic")
    m = _models(G, g, np.float64)
    m.A = A64.astype(np.float64)
    Uf = G["k_Uf"].copy()
    Uc = G["k_Uc"].copy()
    O.step(g, m, Uf, Uc, dtype=np.float64)
    # the current field is damped in place exactly like AbsorbingBoundary
    assert rel(Uc, G["k_damped"]) < 1e-14
    # the new field gets the same per-cell factor on top of the undamped update
    fac = np.divide(G["k_damped"], G["k_Uc"], out=np.ones_like(Uc), where=G["k_Uc"] != 0)
    assert rel(Uf, G["k_acoustic"] * fac) < 1e-12


def _to_full(G, pref):
    nz, nx, N = int(G["k_nz"]), int(G["k_nx"]), int(G["k_N"])
    px = np.zeros((nz, nx)); pz = np.zeros((nz, nx)); zx = np.zeros((nz, nx)); zz = np.zeros((nz, nx))
    px[:, 4:N] = G[pref + "PsixFL"][:, 4:N]
    px[:, nx - N:nx - 4] = G[pref + "PsixFR"][:, 0:N - 4]
    zx[:, 4:N] = G[pref + "ZetaxFL"][:, 4:N]
    zx[:, nx - N:nx - 4] = G[pref + "ZetaxFR"][:, 0:N - 4]
    pz[4:N, :] = G[pref + "PsizFU"][4:N, :]
    pz[nz - N:nz - 4, :] = G[pref + "PsizFD"][0:N - 4, :]
    zz[4:N, :] = G[pref + "ZetazFU"][4:N, :]
    zz[nz - N:nz - 4, :] = G[pref + "ZetazFD"][0:N - 4, :]
    return [px, zx, pz, zz]


@pytest.mark.parametrize("approx,key", [("acoustic", "k_acoustic_cpml"), ("VTI", "k_vti_cpml")])
def test_cpml_step(golden, approx, key):
    G = golden
    g = _grid(G, approx, "CPML")
    m = _models(G, g, np.float64)
    ab = O.cpml_profiles(G["k_vp"], g.N, g.dx, g.dz, g.dt, g.fcut)
    # constants of src/Modeling2D.py:110-126
    R = 1e-3 ** (g.N / 10)
    assert abs(-3 * np.log(R) - float(G["k_d0"])) < 1e-12
    assert abs(g.fcut / 3 - float(G["k_fpico"])) < 1e-12
    m.cpml = ab
    mem = _to_full(G, "k_in_")
    Uf = G["k_Uf"].copy()
    Uc = G["k_Uc"].copy()
    O.step(g, m, Uf, Uc, mem=mem, dtype=np.float64)
    want = _to_full(G, "k_out_")
    for got, exp in zip(mem, want):
        assert rel(got, exp) < 1e-12
    assert rel(Uf, G[key]) < 1e-12


@pytest.mark.parametrize("approx,key", [("VTI", "k_adj_vti"), ("TTI", "k_adj_tti")])
def test_adjoint_imaging_operator(golden, approx, key):
    G = golden
    g = _grid(G, approx)
    m = _models(G, g, np.float64)
    L = O.lib()
    nz, nx = g.nz_a, g.nx_a
    prods = [np.zeros((nz, nx)) for _ in range(5)]
    Uf = G["k_Uf"].copy()
    Uc = G["k_Uc"].copy()
    P = G["k_P"].copy()
    a = O.APPROX[approx]
    p = O._p
    L.og_adjoint_products_f64(a, nz, nx, g.dz, g.dx, p(Uc), p(P), p(m.eps), p(m.delta), p(m.theta),
                              p(prods[0]), p(prods[1]), p(prods[2] if a == 2 else None), p(prods[3]), p(prods[4]))
    img = np.zeros((g.nz, g.nx)); ilum = np.zeros((g.nz, g.nx))
    L.og_rtm_step_f64(a, nz, nx, g.N, g.dz, g.dx, g.dt, p(Uf), p(Uc), p(P), p(img), p(ilum), p(m.vp),
                      *[p(x) for x in prods], None, None, None, None, None, None, None, None, None)
    assert rel(Uf, G[key]) < 1e-12
    N = g.N
    assert rel(img, (Uc * P)[N:nz - N, N:nx - N]) < 1e-14
    assert rel(ilum, (P * P)[N:nz - N, N:nx - N]) < 1e-14


def test_mute(golden):
    G = golden
    got = O.mute(G["m_seis"], G["m_rec_x"], G["m_rec_z"], G["m_shot_x"][1], G["m_shot_z"][1],
                 float(G["m_dt"]), float(G["m_shift"]), float(G["m_window"]), float(G["m_v0"]))
    assert rel(got, G["m_muted"]) < 1e-6


@pytest.mark.parametrize("approx,abc", [("acoustic", "cerjan"), ("acoustic", "CPML"), ("VTI", "cerjan"),
                                        ("VTI", "CPML"), ("TTI", "cerjan")])
def test_time_loop(golden, approx, abc):
    """Full shot loops (injection, step, boundary, recording) against the
    reference wavefield driver src/Modeling2D.py:388-421."""
    G = golden
    pre = f"loop_{approx}_{abc}_"
    g = O.Grid(nz=int(G[pre + "nz"]), nx=int(G[pre + "nx"]), N=int(G[pre + "N"]),
               dz=float(G[pre + "dz"]), dx=float(G[pre + "dx"]), dt=float(G[pre + "dt"]),
               nt=int(G[pre + "nt"]), itlag=int(G[pre + "itlag"]), fcut=float(G[pre + "fcut"]),
               approx=approx, abc=abc)
    N = g.N
    # ExpandModel stores the padded models as float32 (src/Modeling2D.py:42)
    ex = lambda a: O.expand_model(a, N).astype(np.float32).astype(np.float64)
    m = O.Models(vp=ex(G[pre + "vp"]), eps=ex(G[pre + "eps"]), delta=ex(G[pre + "delta"]),
                 theta=ex(G[pre + "theta"]))
    if abc == "CPML":
        m.cpml = O.cpml_profiles(m.vp, N, g.dx, g.dz, g.dt, g.fcut)
    else:
        sb = 3.0 * N
        m.A = np.exp(-((N - np.arange(N)) / (1.4142 * sb)) ** 2)
    seis = O.forward_shot(g, m, G[pre + "src"], int(G[pre + "sx"]), int(G[pre + "sz"]),
                          G[pre + "rx"], G[pre + "rz"], dtype=np.float64)
    assert rel(seis, G[pre + "seis"]) < 1e-11
    # the FP32 oracle (reference C++ order) stays within single-precision accuracy
    seis32 = O.forward_shot(g, m, G[pre + "src"], int(G[pre + "sx"]), int(G[pre + "sz"]),
                            G[pre + "rx"], G[pre + "rz"], dtype=np.float32)
    assert rel(seis32, G[pre + "seis"]) < 1e-4


def test_multiparameter_gradient_terms(golden):
    """The epsilon / delta / theta gradient increments of src/utils.py:1309-1463
    (the VTI vectors come from the reference's TTI function at theta = 0: its
    VTI function cannot run, see tests/golden/make_golden.py)."""
    g = golden
    dx, dz = float(g["k_dx"]), float(g["k_dz"])
    e, d, t = O.multiparameter_gradient_terms(g["mp_cur"], g["mp_adj"], g["k_eps"], g["k_delta"], None, dx, dz)
    assert t is None
    assert rel(e, g["mp_vti_eps"]) < 1e-12 and rel(d, g["mp_vti_delta"]) < 1e-12
    e, d, t = O.multiparameter_gradient_terms(g["mp_cur"], g["mp_adj"], g["k_eps"], g["k_delta"], g["k_theta"], dx,
                                              dz)
    assert rel(e, g["mp_tti_eps"]) < 1e-12 and rel(d, g["mp_tti_delta"]) < 1e-12
    assert rel(t, g["mp_tti_theta"]) < 1e-12
