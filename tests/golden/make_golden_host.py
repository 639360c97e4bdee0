"""Generate the golden fixture of the reference's own host routines.

Builds the reference's cpp/Migration.cu and cpp/Modeling.cu, unmodified, with
the host harness oracle/ref_host.cpp (recipe: oracle/build.py,
``build_ref_host``), runs on small seeded inputs
- Migration::createMask + Migration::smoothModel (cpp/Migration.cu:131-236),
  every field with the water mask of the unsmoothed velocity, as
  Migration::setModel smooths vp, epsilon, delta and theta
  (cpp/Migration.cu:265-290);
- Migration::Mute (cpp/Migration.cu:86-115);
- Modeling::checkDispersionAndStability (cpp/Modeling.cu:184-327), whose
  report is printed with 9 significant digits so every limit is exact;
- Modeling::expandModel (cpp/Modeling.cu:130-182);
and stores inputs and outputs in ``tests/golden/golden_host.npz``.

Usage (needs the reference checkout, so it runs in the development container
only; the fixture it writes is committed):

    python tests/golden/make_golden_host.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# smoothing: (name, field, sigma, parameter)
SMOOTH = [
    ("vp_s0.7", "vp", 0.7, False),
    ("vp_s2.0", "vp", 2.0, False),
    ("vp_s4.5", "vp", 4.5, False),
    ("vp_s12", "vp", 12.0, False),          # 73 taps: wider than the 53-cell rows
    ("eps_s3.0", "eps", 3.0, True),         # eps has zeros below the water too
    ("delta_s6.5", "delta", 6.5, True),
    ("theta_s2.5", "theta", 2.5, True),
]
# mute: (name, nt, nrec, dt, v0, shift, window, shot_x, shot_z)
MUTE = [
    ("m_surface", 300, 41, 0.004, 1500.0, 0.02, 0.03, 1234.5, 10.0),
    ("m_long", 501, 60, 0.002, 1480.0, 0.15, 0.2, 2000.0, 20.0),
    ("m_no_taper", 64, 7, 0.0005, 2000.0, 0.0, 0.0, 0.0, 0.0),
]
# stability: (name, approximation, dx, dz, dt, fcut); the last two fail it
STABILITY = [
    ("s_acoustic", "acoustic", 8.0, 9.0, 6e-4, 12.0),
    ("s_vti", "VTI", 8.0, 9.0, 6e-4, 12.0),
    ("s_tti", "TTI", 8.0, 9.0, 6e-4, 12.0),
    ("s_vti_dt", "VTI", 8.0, 9.0, 2e-3, 12.0),
    ("s_tti_dx", "TTI", 40.0, 40.0, 1e-4, 30.0),
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
    if ob.build_ref_host(force=True, ref_src=os.path.join(ref_root, "cpp")) is None:
        raise SystemExit(f"reference sources not found under {ref_root}/cpp")
    m = models()
    out = {f"in_{k}": v for k, v in m.items()}
    for name, field, sigma, parameter in SMOOTH:
        out[f"out_{name}"] = R.smooth_model(m[field], sigma, parameter, water_model=m["vp"])
    out["smooth_cases"] = np.array([f"{n}|{f}|{s}|{int(p)}" for n, f, s, p in SMOOTH])
    rng = np.random.default_rng(7)
    for name, nt, nrec, dt, v0, shift, window, sx, sz in MUTE:
        seis = rng.standard_normal((nt, nrec)).astype(np.float32)
        rx = np.linspace(0.0, 4000.0, nrec).astype(np.float32)
        rz = np.full(nrec, 20.0, np.float32)
        out[f"{name}_in"], out[f"{name}_rx"], out[f"{name}_rz"] = seis, rx, rz
        out[f"{name}_out"] = R.mute(seis, rx, rz, sx, sz, dt, v0, shift, window)
    out["mute_cases"] = np.array(["|".join(map(str, c)) for c in MUTE])
    for name, approx, dx, dz, dt, fcut in STABILITY:
        args = {"acoustic": (m["vp"],), "VTI": (m["vp"], m["eps"], m["delta"]),
                "TTI": (m["vp"], m["eps"], m["delta"], m["theta"])}[approx]
        r = R.stability(approx, *args, dx=dx, dz=dz, dt=dt, fcut=fcut)
        out[f"{name}_limits"] = np.array([r["dt_lim"], r["dx_lim"], r["dz_lim"]], np.float32)
        out[f"{name}_satisfied"] = np.array(r["satisfied"])
    out["stability_cases"] = np.array(["|".join(map(str, c)) for c in STABILITY])
    out["pad_vp_N50"] = R.expand_model(m["vp"], 50)
    out["pad_theta_N8"] = R.expand_model(m["theta"], 8)
    path = os.path.join(HERE, "golden_host.npz")
    np.savez_compressed(path, **out)
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
