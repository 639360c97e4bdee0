"""Forward modelling on the GPU against the CPU oracle.

Bar: FP32 seismograms within relative L2 1e-5 of the FP32 oracle (the
reference C++ term order, cpp/Modeling.cu:499-749) and of the FP64 oracle.

The VTI/TTI operator of the reference is badly conditioned in FP32: its Sd
term is num/den with den ~ |grad U|^4, switched on only where |den| > 1e-12
(cpp/Modeling.cu:605-611).  The ratio's derivative grows like 1/|grad U| near
amplitude zeros, and at the reference's source scaling (1/(dx dz),
cpp/Modeling.cu:89) the 1e-12 threshold line sweeps through the wavefield, so
a last-bit difference can move a cell across it.  Two FP32 evaluations of the
same formula therefore differ by O(1e-5): measured here, the FP32 oracle (the
reference term order) departs from the FP64 oracle by up to 1.7e-5.  The
anisotropic cases are checked against that yardstick: the GPU's error against
FP64 must stay within max(1e-5, 3 x the FP32 oracle's own error against FP64).
With the Sd term removed (delta = epsilon) they meet the plain 1e-5 bar.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import engine_for, make_case, oracle_models, rel

pytestmark = pytest.mark.gpu

TOL = 1e-5     # relative L2, well-conditioned cases (acoustic; anisotropic with Sd removed)
FP32_FACTOR = 3.0   # anisotropic cases: GPU error vs FP64 <= max(TOL, FP32_FACTOR x FP32-oracle error vs FP64)

CASES = [("acoustic", "cerjan"), ("acoustic", "CPML"), ("VTI", "cerjan"), ("VTI", "CPML"),
         ("TTI", "cerjan"), ("TTI", "CPML")]
ANISO = [c for c in CASES if c[0] != "acoustic"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


def _oracle_seis(case, dtype):
    g = case["grid"]
    m = oracle_models(case)
    return np.stack([O.forward_shot(g, m, case["wavelet"], int(sx), int(sz), case["rx"], case["rz"], dtype=dtype)
                     for sx, sz in zip(case["sx"], case["sz"])])


def _compare(case, label):
    e = engine_for(case)
    seis = e.forward(case["sz"], case["sx"])
    ref32 = _oracle_seis(case, np.float32)
    ref64 = _oracle_seis(case, np.float64)
    assert np.isfinite(seis).all()
    assert np.abs(ref64).max() > 0
    e32, e64, o = rel(seis, ref32), rel(seis, ref64), rel(ref32, ref64)
    print(f"{label}: rel L2 vs FP32 oracle {e32:.2e}, vs FP64 oracle {e64:.2e} (FP32 oracle vs FP64 {o:.2e})")
    return e32, e64, o


@pytest.mark.parametrize("approx,abc", [("acoustic", "cerjan"), ("acoustic", "CPML")])
def test_forward_acoustic(approx, abc):
    e32, e64, _ = _compare(make_case(approx, abc), f"{approx}/{abc}")
    assert e32 < TOL and e64 < TOL


@pytest.mark.parametrize("approx,abc", ANISO)
def test_forward_anisotropic_sd_removed(approx, abc):
    e32, e64, _ = _compare(make_case(approx, abc, sd_off=True), f"{approx}/{abc} Sd removed")
    assert e32 < TOL and e64 < TOL


@pytest.mark.parametrize("amp", [1.0, 1e6])
@pytest.mark.parametrize("approx,abc", ANISO)
def test_forward_anisotropic(approx, abc, amp):
    """Reference amplitude (threshold sweeping the field) and x1e6 (Sd on
    almost everywhere)."""
    e32, e64, o = _compare(make_case(approx, abc, amp=amp), f"{approx}/{abc} amplitude x{amp:g}")
    assert e64 < max(TOL, FP32_FACTOR * o)


@pytest.mark.parametrize("approx,abc", [("acoustic", "cerjan"), ("TTI", "CPML")])
def test_batch_equals_single_shots(approx, abc):
    """A shot's result does not depend on the batch it runs in (bitwise)."""
    case = make_case(approx, abc, nshots=4, seed=3)
    e = engine_for(case)
    batch = e.forward(case["sz"], case["sx"])
    for i in range(4):
        one = e.forward(case["sz"][i:i + 1], case["sx"][i:i + 1])
        assert np.array_equal(one[0], batch[i])


@pytest.mark.parametrize("approx,abc", [("VTI", "CPML"), ("acoustic", "cerjan")])
def test_autotuned_tile_height_is_bitwise_neutral(approx, abc, monkeypatch):
    """The segment-height tuner of the graph path picks one of its candidates
    per batch size, and the seismograms are bitwise those of the default
    height.  (Small Cerjan runs otherwise take the persistent path, which
    sets its own height.)"""
    monkeypatch.setenv("PAM_NO_PERSISTENT", "1")
    case = make_case(approx, abc, nz=150, nx=130, nshots=3, seed=11)
    fixed = engine_for(case)
    fixed.autotune(False)
    ref = fixed.forward(case["sz"], case["sx"])
    assert fixed.segment_height(3) == 0
    tuned = engine_for(case)
    out = tuned.forward(case["sz"], case["sx"])
    h = tuned.segment_height(3)
    print(f"{approx}/{abc}: tuned segment height {h}")
    assert h in (8, 16, 24, 32, 48, 64, 96, 128)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("approx", ["acoustic", "VTI", "TTI"])
def test_persistent_time_loop_is_bitwise_the_graph(approx, monkeypatch):
    """Small Cerjan runs go through one cooperative launch per time chunk
    (a grid-wide barrier between steps, one-row segments); their seismograms,
    host and device paths, are bitwise those of the graph of one-step
    launches (PAM_NO_PERSISTENT) and of one launch per kernel and step
    (PAM_NO_GRAPH)."""
    import torch
    case = make_case(approx, "cerjan", nshots=2, seed=5)
    e = engine_for(case)
    persistent = e.forward(case["sz"], case["sx"])
    dev = torch.empty((2, e.cfg.nt_data, len(case["rx"])), dtype=torch.float32, device="cuda")
    e.forward_device(torch.as_tensor(case["sz"], dtype=torch.int32, device="cuda"),
                     torch.as_tensor(case["sx"], dtype=torch.int32, device="cuda"), dev)
    torch.cuda.synchronize()
    monkeypatch.setenv("PAM_NO_PERSISTENT", "1")
    graph = e.forward(case["sz"], case["sx"])
    monkeypatch.setenv("PAM_NO_GRAPH", "1")
    per_launch = e.forward(case["sz"], case["sx"])
    print(f"{approx}: persistent vs graph max |diff| {np.abs(persistent - graph).max():.3e}")
    assert np.isfinite(persistent).all() and np.abs(persistent).max() > 0
    assert np.array_equal(persistent, graph) and np.array_equal(graph, per_launch)
    assert np.array_equal(dev.cpu().numpy(), persistent)


def test_step_interface_wavefield():
    """pam_begin / pam_step / pam_read_wavefield follow the reference loop:
    after step k the current field is U(k+1) with source k+1 injected."""
    case = make_case("VTI", "cerjan", nt=150, nshots=2, seed=5, sd_off=True)
    g = case["grid"]
    e = engine_for(case)
    e.begin(case["sz"], case["sx"])
    for k in range(g.nt):
        e.step(k)
    u_gpu = e.read_wavefield(1)
    seis = e.read_seismograms()
    m = oracle_models(case)
    fields = {}

    def grab(k, st):
        if k == g.nt - 1:
            fields["U"] = st.fut.copy()   # U(nt) before the swap

    ref = O.forward_shot(g, m, case["wavelet"], int(case["sx"][1]), int(case["sz"][1]), case["rx"], case["rz"],
                         dtype=np.float32, on_step=grab)
    assert rel(seis[1], ref) < TOL
    # the engine keeps U(t-1) undamped in storage and applies the Cerjan factor
    # when it is read; compare the interior, where both agree
    N = g.N
    assert rel(u_gpu[N:-N, N:-N], fields["U"][N:-N, N:-N]) < TOL


def test_forward_device_path_matches_host_path():
    torch = pytest.importorskip("torch")
    case = make_case("acoustic", "CPML", seed=7)
    e = engine_for(case)
    host = e.forward(case["sz"], case["sx"])
    dsz = torch.tensor(case["sz"], dtype=torch.int32, device="cuda")
    dsx = torch.tensor(case["sx"], dtype=torch.int32, device="cuda")
    out = torch.empty((3, case["grid"].nt_data, case["rx"].size), dtype=torch.float32, device="cuda")
    e.forward_device(dsz, dsx, out, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


def test_pinned_output_streams_the_seismograms_during_the_loop():
    """A pinned output buffer makes pam_forward run the time loop as a chain of
    graphs over time chunks and copy each chunk's samples while the next one
    computes; the result must equal the single copy into pageable memory, for a
    full and a partial batch, on the engine's stream and on a caller's stream,
    and after switching back and forth between the paths."""
    torch = pytest.importorskip("torch")
    case = make_case("VTI", "CPML", seed=8, sd_off=True)
    e = engine_for(case)
    g = case["grid"]
    nrec = case["rx"].size
    ref = e.forward(case["sz"], case["sx"])
    pinned = torch.empty((3, g.nt_data, nrec), dtype=torch.float32).pin_memory()
    out = e.forward(case["sz"], case["sx"], out=pinned.numpy())
    assert np.array_equal(out, ref)
    st = torch.cuda.Stream()
    pinned.zero_()
    e.forward(case["sz"], case["sx"], out=pinned.numpy(), stream=st.cuda_stream)
    assert np.array_equal(pinned.numpy(), ref)
    part = torch.zeros((2, g.nt_data, nrec), dtype=torch.float32).pin_memory()
    e.forward(case["sz"][1:], case["sx"][1:], out=part.numpy())
    assert np.array_equal(part.numpy(), e.forward(case["sz"][1:], case["sx"][1:]))
    assert np.array_equal(e.forward(case["sz"], case["sx"]), ref)


def test_unstable_time_step_is_reported():
    """A time step ten times beyond the stability limit overflows the fields to
    inf / NaN within a few dozen steps (plain float arithmetic; no index
    depends on the data): modelling reports PAM_E_NUMERIC, and so does the
    gradient job through its misfit."""
    from pseudoacousticmodeling_gb300 import PamError
    case = make_case("acoustic", "cerjan", nt=300, seed=3, dt=0.01)
    e = engine_for(case)
    with pytest.raises(PamError, match="PAM_E_NUMERIC: non-finite values in the seismograms"):
        e.forward(case["sz"], case["sx"])
    dobs = np.zeros((len(case["sx"]), case["grid"].nt_data, case["rx"].size), np.float32)
    with pytest.raises(PamError, match="PAM_E_NUMERIC: non-finite misfit"):
        e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=0)
    stable = engine_for(make_case("acoustic", "cerjan", nt=300, seed=3))
    assert np.isfinite(stable.forward(case["sz"], case["sx"])).all()


def test_bad_arguments_raise():
    from pseudoacousticmodeling_gb300 import PamError
    case = make_case("acoustic", "cerjan", nshots=1)
    e = engine_for(case)
    with pytest.raises(PamError):
        e.forward(np.array([0], np.int32), np.array([5], np.int32))   # source in the frame
    with pytest.raises(PamError):
        e.forward(np.array([30, 30], np.int32), np.array([40, 50], np.int32))   # more shots than max_shots
    with pytest.raises(PamError):
        e.set_receivers(np.array([10_000], np.int32), np.array([5], np.int32))
