"""The C ABI without a GPU: the library loads, exports every function that
include/pam.h declares (each also bound by the Python layer), fails cleanly
where a device is needed, and its host-only utilities work."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pam.h")


@pytest.fixture(scope="module")
def lib():
    from pseudoacousticmodeling_gb300 import _lib, build
    build.build()
    return _lib.load()


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(pam_\w+)\s*\(", text, re.M)))


def test_every_declared_function_is_exported_and_bound(lib):
    from pseudoacousticmodeling_gb300 import _lib
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/pam.h but not exported"
        assert n in _lib.SIGNATURES, f"{n} not bound in _lib.SIGNATURES"
    assert set(_lib.SIGNATURES) <= set(names)


def _prototypes():
    """name -> list of parameter declarations, from the prototypes of include/pam.h."""
    text = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"(?:const\s+)?\w+\s*\*?\s*(pam_\w+)\s*\(([^)]*)\)\s*;", text):
        params = [q.strip() for q in m.group(2).split(",") if q.strip()]
        out[m.group(1)] = [] if params == ["void"] else params
    return out


def test_bindings_match_the_prototypes():
    """Every binding in _lib.SIGNATURES has the header prototype's parameter
    count, a pointer where the prototype takes a pointer, and the same scalar
    type where it takes a value."""
    from pseudoacousticmodeling_gb300 import _lib
    protos = _prototypes()
    assert set(protos) == set(_declared())
    scalars = {"int": (ctypes.c_int, ctypes.c_int32), "float": (ctypes.c_float,), "double": (ctypes.c_double,),
               "long long": (ctypes.c_longlong, ctypes.c_int64),
               "unsigned long long": (ctypes.c_ulonglong, ctypes.c_uint64), "size_t": (ctypes.c_size_t,)}
    for name, (_, argtypes) in _lib.SIGNATURES.items():
        params = protos[name]
        assert len(params) == len(argtypes), f"{name}: {len(params)} parameters declared, {len(argtypes)} bound"
        for decl, t in zip(params, argtypes):
            if "*" in decl:
                assert t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and \
                    issubclass(t, ctypes._Pointer), f"{name}: '{decl}' bound as {t}"
            else:
                base = " ".join(w for w in decl.split()[:-1] if w != "const")
                assert t in scalars.get(base, ()), f"{name}: '{decl}' bound as {t}"


def test_create_without_a_device_fails_cleanly(lib):
    from pseudoacousticmodeling_gb300 import Config, Engine, PamError
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(PamError):
        Engine(Config(nz=20, nx=20, n_abc=10, dz=10.0, dx=10.0, dt=0.001, nt=50, itlag=10, fcut=20.0,
                      approximation="acoustic", boundary="cerjan", max_shots=1))


def _random_boundary(lib, vp, N, dvel=1000.0, ratio=200.0, vcap=6000.0, seed=0, h=10.0):
    nz, nx = vp.shape
    out = np.zeros((nz + 2 * N, nx + 2 * N), np.float32)
    vp = np.ascontiguousarray(vp, np.float32)
    n = lib.pam_random_boundary(vp.ctypes.data_as(ctypes.c_void_p), nz, nx, N, h, h, dvel, ratio, vcap, seed,
                                out.ctypes.data_as(ctypes.c_void_p))
    return n, out


def test_random_boundary_generator(lib):
    rng = np.random.default_rng(0)
    nz, nx, N = 60, 90, 30
    vp = (1800.0 + 400.0 * rng.random((nz, nx))).astype(np.float32)
    n, a = _random_boundary(lib, vp, N, seed=7)
    n2, b = _random_boundary(lib, vp, N, seed=7)
    _, c = _random_boundary(lib, vp, N, seed=8)
    assert n > 0 and n == n2 and np.array_equal(a, b)          # deterministic for a seed
    assert not np.array_equal(a, c)
    assert np.array_equal(a[N:N + nz, N:N + nx], vp)            # the interior is untouched
    border = np.ones_like(a, bool)
    border[N:N + nz, N:N + nx] = False
    lo, hi = max(1.0, vp.min() - 1000.0), min(vp.max() + 1000.0, 6000.0)
    assert a[border].min() >= lo - 1e-3 and a[border].max() <= hi + 1e-3
    # random: the border is no longer the edge replication of the model
    edge = np.pad(vp, N, mode="edge")
    assert np.abs(a[border] - edge[border]).mean() > 50.0
    # the stability cap holds
    _, d = _random_boundary(lib, vp, N, vcap=2300.0)
    assert d[border].max() <= 2300.0 + 1e-3
    # invalid arguments
    bad, _ = _random_boundary(lib, vp, N, ratio=0.0)
    assert bad == -1


def test_bounds_checked_build_compiles_and_exports_the_abi():
    """The check build (-DPAM_BOUNDS_CHECK, used by the GPU memory-safety test)
    compiles here and exports every entry point of include/pam.h."""
    from pseudoacousticmodeling_gb300 import build
    lib = ctypes.CDLL(build.build_checked())
    for n in _declared():
        assert hasattr(lib, n), f"{n} missing from the checked build"
