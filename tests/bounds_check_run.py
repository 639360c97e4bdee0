"""Run a set of small modelling, migration and gradient jobs with the library
given on the command line and print one JSON object of exact checksums.

Used by tests/test_gpu_bounds_check.py, once with the normal library and once
with the bounds-checked one (-DPAM_BOUNDS_CHECK), each in a process of its
own: the checked kernels print "PAM_BOUNDS ..." for any access outside its
buffer, and the checksums of the two builds must be equal."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

from pseudoacousticmodeling_gb300 import _lib  # noqa: E402

_lib.load(sys.argv[1])

from pseudoacousticmodeling_gb300 import Config, Engine  # noqa: E402
from tests.gpu_cases import engine_for, make_case  # noqa: E402


def csum(a):
    a = np.asarray(a, np.float64)
    return [float(a.sum()), float(np.abs(a).sum())]


out = {}
for approx in ("acoustic", "VTI", "TTI"):
    for abc in ("cerjan", "CPML"):
        key = f"{approx}/{abc}"
        # odd width, receivers on the update region's edges, a source in the border
        case = make_case(approx, abc, nz=61, nx=133, N=12, nt=150, nshots=3, seed=41, sd_off=(approx != "acoustic"))
        g = case["grid"]
        case["sx"] = np.array([5, g.nx_a // 2, g.nx_a - 6], np.int32)
        case["sz"] = np.array([g.N + 1, 6, g.nz_a - 7], np.int32)
        e = engine_for(case)
        # per-shot receiver spreads (the most receivers first: the engine sizes
        # its seismogram buffer at the first modelling call)
        rxs = np.stack([np.clip(int(s) - 20 + 3 * np.arange(9), 4, g.nx_a - 5) for s in case["sx"]]).astype(np.int32)
        rzs = np.stack([np.full(9, g.N + 2 + b, np.int32) for b in range(3)])
        e.set_receivers(rzs, rxs, per_shot=True)
        out[key + " forward per-shot"] = csum(e.forward(case["sz"], case["sx"]))
        # receivers on the corners of the update region and one in the middle
        rx = np.array([4, g.nx_a - 5, 4, g.nx_a - 5, g.nx_a // 2], np.int32)
        rz = np.array([4, 4, g.nz_a - 5, g.nz_a - 5, g.N + 1], np.int32)
        e.set_receivers(rz, rx)
        seis = e.forward(case["sz"], case["sx"])
        out[key + " forward"] = csum(seis)
        if approx != "acoustic" and abc == "CPML":   # anisotropic migration and FWI are Cerjan-only
            e.close()
            continue
        # migration with every source-field strategy
        for K in (0, 17, -1, -2):
            if K == -2:
                e.set_random_boundary(dvel=500.0, ratio=40.0, seed=2)
            e.rtm_reset()
            e.rtm(case["sz"], case["sx"], seis, ckpt_interval=K)
            out[f"{key} rtm K={K}"] = csum(e.rtm_result(norm="none")[0])
        # gradients: the exact one (acoustic Cerjan), the reference form (all)
        dobs = 1.01 * seis
        if approx == "acoustic" and abc == "cerjan":
            for K in (0, 23):
                J, gvp = e.misfit_gradient(case["sz"], case["sx"], dobs, ckpt_interval=K)
                out[f"{key} exact gradient K={K}"] = [J] + csum(gvp)
        if approx != "acoustic":
            e.set_multiparameter(True)
        e.rtm_reset()
        J = e.fwi_gradient(case["sz"], case["sx"], dobs, ckpt_interval=19)
        out[key + " reference gradient"] = [J] + csum(e.fwi_result()[0])
        if approx != "acoustic":
            out[key + " multiparameter"] = sum((csum(x) for x in e.fwi_multiparameter_result() if x is not None), [])
        e.close()
# the smallest grid the engine accepts
for abc in ("cerjan", "CPML"):
    e = Engine(Config(nz=8, nx=8, n_abc=8, dz=10.0, dx=10.0, dt=0.001, nt=120, itlag=30, fcut=30.0,
                      approximation="acoustic", boundary=abc, max_shots=1))
    e.set_models(np.repeat(np.linspace(1600.0, 2000.0, 8, dtype=np.float32)[:, None], 8, axis=1))
    e.set_receivers(np.full(8, 8, np.int32), np.arange(8, 16, dtype=np.int32))
    out[f"8x8 {abc}"] = csum(e.forward(np.array([9], np.int32), np.array([10], np.int32)))
    e.close()
# the allocation-free misfit, with a sample count that is not a multiple of
# its 2,048-sample blocks (the last block reads a partial range)
import ctypes  # noqa: E402

import torch  # noqa: E402

lib = _lib.load()
rng = np.random.default_rng(3)
n = 3 * 2048 + 777
dcal = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
dobs = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
mis = ctypes.c_double(0.0)
rc = lib.pam_misfit_noalloc(ctypes.c_void_p(dcal.data_ptr()), ctypes.c_void_p(dobs.data_ptr()), n,
                            ctypes.byref(mis), None)
assert rc == 0, rc
out["misfit_noalloc odd n"] = [mis.value]
print("CHECKSUMS " + json.dumps(out))
