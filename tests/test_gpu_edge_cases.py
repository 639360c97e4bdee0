"""Edge cases of the forward and migration paths against the CPU oracle:
per-shot receiver spreads (cpp/Survey.cpp geometry per shot), receivers on
the first and last updated rows and columns, a single receiver, a source
inside the absorbing border, the smallest grid the engine accepts, and a
batch smaller than the engine's capacity."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import engine_for, make_case, oracle_models, rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


def _oracle(case, m, sx, sz, rx, rz):
    return O.forward_shot(case["grid"], m, case["wavelet"], int(sx), int(sz), rx, rz, dtype=np.float32)


@pytest.mark.parametrize("abc", ["cerjan", "CPML"])
def test_per_shot_receiver_spreads(abc):
    case = make_case("acoustic", abc, nshots=3, seed=31)
    g = case["grid"]
    nrec = 25
    rx = np.stack([np.clip(int(sx) - 30 + 3 * np.arange(nrec), 4, g.nx_a - 5) for sx in case["sx"]]).astype(np.int32)
    rz = np.stack([np.full(nrec, g.N + 2 + b, np.int32) for b in range(3)])
    e = engine_for(case)
    e.set_receivers(rz, rx, per_shot=True)
    seis = e.forward(case["sz"], case["sx"])
    m = oracle_models(case)
    ref = np.stack([_oracle(case, m, case["sx"][b], case["sz"][b], rx[b], rz[b]) for b in range(3)])
    err = rel(seis, ref)
    print(f"per-shot receiver spreads ({abc}): {err:.2e}")
    assert seis.shape == (3, g.nt_data, nrec) and err < TOL
    # migration with the same spreads: the sum of the oracle's per-shot images
    e.rtm(case["sz"], case["sx"], ref, ckpt_interval=0)
    img, _ = e.rtm_result(norm="none")
    r_img = sum(O.rtm_shot(g, m, case["wavelet"], int(case["sx"][b]), int(case["sz"][b]), rx[b], rz[b], ref[b],
                           dtype=np.float32)[0] for b in range(3))
    assert rel(img, r_img) < 1e-4


def test_receivers_on_the_update_region_edges_and_a_single_receiver():
    case = make_case("VTI", "cerjan", nshots=2, seed=32, sd_off=True)
    g = case["grid"]
    rx = np.array([4, g.nx_a - 5, 4, g.nx_a - 5, g.nx_a // 2], np.int32)
    rz = np.array([4, 4, g.nz_a - 5, g.nz_a - 5, g.N + 1], np.int32)
    e = engine_for(case)
    e.set_receivers(rz, rx)
    seis = e.forward(case["sz"], case["sx"])
    m = oracle_models(case)
    ref = np.stack([_oracle(case, m, sx, sz, rx, rz) for sx, sz in zip(case["sx"], case["sz"])])
    assert rel(seis, ref) < TOL
    e.set_receivers(rz[-1:], rx[-1:])
    one = e.forward(case["sz"], case["sx"])
    assert one.shape == (2, g.nt_data, 1)
    assert np.array_equal(one[:, :, 0], seis[:, :, -1])


def test_source_inside_the_absorbing_border():
    case = make_case("acoustic", "cerjan", nshots=2, seed=33)
    g = case["grid"]
    case["sx"] = np.array([5, g.nx_a - 6], np.int32)
    case["sz"] = np.array([6, g.nz_a - 7], np.int32)
    e = engine_for(case)
    seis = e.forward(case["sz"], case["sx"])
    m = oracle_models(case)
    ref = np.stack([_oracle(case, m, sx, sz, case["rx"], case["rz"]) for sx, sz in zip(case["sx"], case["sz"])])
    assert np.abs(ref).max() > 0
    assert rel(seis, ref) < TOL


@pytest.mark.parametrize("abc", ["cerjan", "CPML"])
def test_smallest_grid(abc):
    """The smallest model the engine accepts: 8 x 8 cells with the smallest
    border (8 cells); a 7-row model is refused (the strips would overlap)."""
    from pseudoacousticmodeling_gb300 import Config, Engine, PamError
    with pytest.raises(PamError, match="overlap"):
        Engine(Config(nz=7, nx=8, n_abc=8, dz=10.0, dx=10.0, dt=0.001, nt=20, itlag=5, fcut=30.0,
                      approximation="acoustic", boundary=abc, max_shots=1))
    nz, nx, N, nt, dt, fcut = 8, 8, 8, 120, 0.001, 30.0
    tlag = 2.0 * np.sqrt(np.pi) / fcut
    g = O.Grid(nz=nz, nx=nx, N=N, dz=10.0, dx=10.0, dt=dt, nt=nt, itlag=int(round(tlag / dt)), fcut=fcut,
               approx="acoustic", abc=abc)
    vp = np.repeat(np.linspace(1600.0, 2000.0, nz, dtype=np.float32)[:, None], nx, axis=1)
    case = dict(grid=g, vp=vp, eps=None, delta=None, theta=None,
                wavelet=O.ricker_cpp(nt, dt, fcut, np.float32(tlag), 10.0, 10.0))
    case["sx"] = np.array([g.N + 2], np.int32)
    case["sz"] = np.array([g.N + 1], np.int32)
    case["rx"] = np.arange(g.N, g.N + g.nx, dtype=np.int32)
    case["rz"] = np.full(g.nx, g.N, np.int32)
    e = engine_for(case)
    seis = e.forward(case["sz"], case["sx"])
    ref = _oracle(case, oracle_models(case), case["sx"][0], case["sz"][0], case["rx"], case["rz"])
    assert np.isfinite(seis).all() and np.abs(ref).max() > 0
    assert rel(seis[0], ref) < TOL


def test_batch_smaller_than_capacity():
    case = make_case("TTI", "CPML", nshots=3, seed=35, sd_off=True)
    full = engine_for(case).forward(case["sz"], case["sx"])
    big = engine_for(case, max_shots=8)
    assert np.array_equal(big.forward(case["sz"], case["sx"]), full)
    assert np.array_equal(big.forward(case["sz"][1:2], case["sx"][1:2])[0], full[1])


@pytest.mark.parametrize("N", [13, 200])
def test_cpml_strip_kernel_variants(N):
    """CPML forward against the oracle for the strip kernels' other forms: an
    odd border (13 cells: the x strips one cell per thread, since pairs need
    even strip-row offsets) and a border taller than 192 strip cells (200: the
    z strips one column per thread, eight rows each)."""
    case = make_case("VTI", "CPML", nz=24, nx=40, N=N, nt=150, nshots=2, seed=44)
    seis = engine_for(case).forward(case["sz"], case["sx"])
    m = oracle_models(case)
    ref = np.stack([_oracle(case, m, sx, sz, case["rx"], case["rz"]) for sx, sz in zip(case["sx"], case["sz"])])
    err = rel(seis, ref)
    print(f"\nCPML border {N}: relative L2 vs FP32 oracle {err:.2e}")
    assert np.isfinite(seis).all() and np.abs(ref).max() > 0 and err < TOL
