"""Generate the golden fixture of the reference's model smoothing.

Builds the reference's own cpp/Migration.cu and cpp/Modeling.cu, unmodified,
with the host harness oracle/ref_smooth.cpp (recipe: oracle/build.py,
``build_ref_smooth``), runs Migration::createMask and Migration::smoothModel
(cpp/Migration.cu:131-236) on small seeded models, and stores inputs and
outputs in ``tests/golden/golden_smooth.npz``.  Every case smooths with the
water mask of the unsmoothed velocity, as Migration::setModel does for vp,
epsilon, delta and theta (cpp/Migration.cu:265-290).

Usage (needs the reference checkout, so it runs in the development container
only; the fixture it writes is committed):

    python tests/golden/make_golden_smooth.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (name, field, sigma, parameter): the field is smoothed with the velocity's mask
CASES = [
    ("vp_s0.7", "vp", 0.7, False),
    ("vp_s2.0", "vp", 2.0, False),
    ("vp_s4.5", "vp", 4.5, False),
    ("vp_s12", "vp", 12.0, False),          # 73 taps: wider than the 53-cell rows
    ("eps_s3.0", "eps", 3.0, True),         # eps has zeros below the water too
    ("delta_s6.5", "delta", 6.5, True),
    ("theta_s2.5", "theta", 2.5, True),
]


def models():
    rng = np.random.default_rng(20261204)
    nz, nx = 37, 53
    vp = np.full((nz, nx), 1480.0, np.float32)                       # water layer: the minimum
    vp[9:] = (1900.0 + 900.0 * rng.random((nz - 9, nx))).astype(np.float32)
    eps = (0.25 * rng.random((nz, nx))).astype(np.float32)
    eps[:9] = 0.0
    eps[20, 5] = 0.0                                                  # eps's own minimum off the water
    delta = (0.1 * rng.random((nz, nx))).astype(np.float32)
    delta[:9] = 0.0
    theta = (-35.0 + 70.0 * rng.random((nz, nx))).astype(np.float32)
    return {"vp": vp, "eps": eps, "delta": delta, "theta": theta}


def main(ref_root):
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    from oracle import ref as R
    lib = ob.build_ref_smooth(force=True, ref_src=os.path.join(ref_root, "cpp"))
    if lib is None:
        raise SystemExit(f"reference sources not found under {ref_root}/cpp")
    m = models()
    out = {f"in_{k}": v for k, v in m.items()}
    for name, field, sigma, parameter in CASES:
        out[f"out_{name}"] = R.smooth_model(m[field], sigma, parameter, water_model=m["vp"])
    out["cases"] = np.array([f"{n}|{f}|{s}|{int(p)}" for n, f, s, p in CASES])
    path = os.path.join(HERE, "golden_smooth.npz")
    np.savez_compressed(path, **out)
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
