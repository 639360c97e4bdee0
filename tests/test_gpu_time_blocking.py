"""Two time steps per launch (pam_set_time_blocking, acoustic with Cerjan
boundaries) against one step per launch.

The two-step kernel repeats the one-step arithmetic operation for operation,
so every result must be bitwise equal: seismograms (device output, and pinned
host output whose time chunks end on odd steps), migration images and exact
gradients with checkpoint intervals that split pairs.  The cases put sources
on the columns that two neighbouring tiles both compute (the kernel's halo
lanes), in the absorbing border and near segment ends."""
import numpy as np
import pytest

from tests.gpu_cases import engine_for, make_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from pseudoacousticmodeling_gb300 import build
    build.build()


def _case(nt, nx=250, nz=70, seed=31):
    case = make_case("acoustic", "cerjan", nz=nz, nx=nx, N=20, nt=nt, nshots=4, seed=seed)
    g = case["grid"]
    # tile seams of the two-step kernel are at columns 120 t .. 120 t + 3
    case["sx"] = np.array([122, 5, 241, g.nx_a // 2 + 1], np.int32)
    case["sz"] = np.array([24, 9, g.nz_a - 6, 68], np.int32)
    return case


@pytest.mark.parametrize("nt,nz,nx", [(231, 70, 250), (260, 70, 250), (201, 157, 371)])
def test_two_step_forward_equals_one_step(nt, nz, nx):
    torch = pytest.importorskip("torch")
    case = _case(nt, nx=nx, nz=nz)
    e = engine_for(case)
    assert e.set_time_blocking(True)
    a = e.forward(case["sz"], case["sx"])
    pinned = torch.empty(a.shape, dtype=torch.float32).pin_memory().numpy()
    e.forward(case["sz"], case["sx"], out=pinned)
    e.set_time_blocking(False)
    b = e.forward(case["sz"], case["sx"])
    print(f"nt={nt} {nz}x{nx}: max |seis| {np.abs(b).max():.3e}, "
          f"differing samples {int((a != b).sum())} / {a.size}")
    assert np.abs(b).max() > 0
    assert np.array_equal(a, b)
    assert np.array_equal(pinned, b)


def test_two_step_gradient_and_migration_equal_one_step():
    case = _case(233)
    e = engine_for(case)
    dobs = (1.02 * e.forward(case["sz"], case["sx"])).astype(np.float32)
    out = {}
    for on in (True, False):
        e.set_time_blocking(on)
        for K in (0, 23, 58):
            out[(on, "grad", K)] = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=K)
        e.rtm_reset()
        e.rtm(case["sz"], case["sx"], dobs, ckpt_interval=17)
        out[(on, "rtm")] = e.rtm_result(norm="none")[0]
    for K in (0, 23, 58):
        a, b = out[(True, "grad", K)], out[(False, "grad", K)]
        assert a[0] == b[0] and np.array_equal(a[1], b[1]), K
    assert np.array_equal(out[(True, "rtm")], out[(False, "rtm")])
    assert np.abs(out[(False, "rtm")]).max() > 0


def test_time_blocking_reports_the_operators_that_have_it():
    for approx, abc, has in (("acoustic", "cerjan", True), ("acoustic", "CPML", False), ("VTI", "cerjan", False)):
        case = make_case(approx, abc, nt=40, nshots=1)
        e = engine_for(case)
        assert e.set_time_blocking(True) == has
        e.close()
