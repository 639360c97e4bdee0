"""End-to-end drop-in: a job in the reference's formats (Parameters.json, CSV
geometry, raw float32 models) through the command-line drivers and through
the reference-shaped Python classes, against the CPU oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import rel

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "pseudoacousticmodeling_gb300", "_build")


@pytest.fixture(scope="module")
def job(tmp_path_factory):
    from pseudoacousticmodeling_gb300 import build
    from pseudoacousticmodeling_gb300.survey import save_bin, write_csv_geometry
    build.build()
    d = tmp_path_factory.mktemp("job")
    for sub in ("models", "seis", "img", "grad"):
        (d / sub).mkdir()
    nz, nx, h = 61, 121, 10.0
    vp = np.full((nz, nx), 1500.0, np.float32)
    vp[25:, :] = 2200.0
    vp[45:, :] = 2700.0
    save_bin(str(d / "models" / "vp.bin"), vp)
    write_csv_geometry(d / "rec.csv", np.arange(0, (nx - 1) * h + 1, 2 * h), np.full((nx + 1) // 2, 20.0))
    write_csv_geometry(d / "src.csv", np.array([200.0, 600.0, 1000.0]), np.full(3, 20.0))
    p = {"unit": "GPU", "approximation": "acoustic", "migration": "checkpoint", "ABC": "cerjan",
         "dx": h, "dz": h, "dt": 0.001, "L": (nx - 1) * h, "D": (nz - 1) * h, "T": 0.4, "N_abc": 20,
         "fcut": 25.0, "sigma": 3.0, "v0": 1500.0, "shift": 0.05, "window": 0.03, "step": 50,
         "rec_file": "rec.csv", "src_file": "src.csv", "vpFile": "models/vp.bin",
         "seismogramFolder": "seis/", "imageFolder": "img/", "gradientsFolder": "grad/",
         "batch": 2, "ckpt_interval": 40}
    (d / "Parameters.json").write_text(json.dumps(p))
    return d, vp


def _run(exe, d):
    r = subprocess.run([os.path.join(BUILD, exe), str(d / "Parameters.json")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_drivers_and_python_classes(job):
    from pseudoacousticmodeling_gb300.migration import migration
    from pseudoacousticmodeling_gb300.modeling import wavefield
    from pseudoacousticmodeling_gb300.survey import import_bin, parameters
    d, vp = job
    pmt = parameters(str(d / "Parameters.json"))
    assert (pmt.nz, pmt.nx, pmt.nt_data, pmt.Nshot, pmt.Nrec) == (61, 121, 401, 3, 61)

    out = _run("pam_modeling", d)
    assert "Run time" in out
    seis_files = [pmt.seismogram_file(s) for s in range(pmt.Nshot)]
    drv = np.stack([import_bin(f, (pmt.nt_data, pmt.Nrec)) for f in seis_files])

    # the reference-shaped Python classes on the same job: bitwise equal
    wf = wavefield(pmt)
    wf.loadModels()
    wf.initializeWavefields()
    wf.setModels()
    assert wf.checkDispersionAndStability()
    py = wf.SolveWaveEquation(save=False)
    assert np.array_equal(py, drv)

    # and the oracle (C++ Ricker, race-free Cerjan)
    g = O.Grid(nz=pmt.nz, nx=pmt.nx, N=pmt.N_abc, dz=pmt.dz, dx=pmt.dx, dt=pmt.dt, nt=pmt.nt, itlag=pmt.itlag,
               fcut=pmt.fcut)
    m = O.Models.build(g, vp)
    w = O.ricker_cpp(pmt.nt, pmt.dt, pmt.fcut, np.float32(pmt.tlag), pmt.dx, pmt.dz)
    ref = np.stack([O.forward_shot(g, m, w, int(sx), int(sz), pmt.rx, pmt.rz, dtype=np.float32)
                    for sx, sz in zip(pmt.sx, pmt.sz)])
    assert rel(drv, ref) < 1e-5

    # migration: driver vs Python class (same engine, same smoothing and mute)
    _run("pam_migration", d)
    img_drv = import_bin(pmt.image_file(), (pmt.nz, pmt.nx))
    mg = migration(wf, pmt)
    img_py, _ = mg.SolveBackwardWaveEquation(save=False)
    assert np.isfinite(img_drv).all() and np.abs(img_drv).max() > 0
    assert rel(img_drv, img_py) < 1e-5

    # gradient driver runs and writes a finite gradient
    _run("pam_inversion", d)
    gr = import_bin(pmt.gradient_file(), (pmt.nz, pmt.nx))
    assert np.isfinite(gr).all()


def test_drivers_shard_shots_over_ranks(job):
    """RANK / WORLD_SIZE split the shots of the drivers: two ranks (run one
    after the other here; on a node, one process per GPU) write their shots'
    seismograms and their partial images and gradients, and --reduce adds the
    partial sums into the files a single process writes."""
    from pseudoacousticmodeling_gb300.survey import import_bin, parameters, save_bin
    d, _ = job
    pmt = parameters(str(d / "Parameters.json"))

    def run_rank(exe, rank, world):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world))
        r = subprocess.run([os.path.join(BUILD, exe), str(d / "Parameters.json")], capture_output=True, text=True,
                           env=env)
        assert r.returncode == 0, r.stdout + r.stderr
        return r.stdout

    env1 = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE")}

    def run_single(exe):
        r = subprocess.run([os.path.join(BUILD, exe), str(d / "Parameters.json")], capture_output=True, text=True,
                           env=env1)
        assert r.returncode == 0, r.stdout + r.stderr

    seis_files = [pmt.seismogram_file(s) for s in range(pmt.Nshot)]
    run_single("pam_modeling")
    seis_single = [import_bin(f, (pmt.nt_data, pmt.Nrec)) for f in seis_files]
    for f in seis_files:
        os.remove(f)
    # modelling: each rank writes its own shots (3 shots over 2 ranks: 2 + 1)
    outs = [run_rank("pam_modeling", r, 2) for r in range(2)]
    assert "Shots 1-2 of 3" in outs[0] and "Shots 3-3 of 3" in outs[1]
    for s in range(pmt.Nshot):
        assert np.array_equal(import_bin(seis_files[s], (pmt.nt_data, pmt.Nrec)), seis_single[s])
    # observed data that differ from the model's own (a non-zero FWI residual)
    for f, d0 in zip(seis_files, seis_single):
        save_bin(f, (1.05 * d0).astype(np.float32))
    single = {}
    for exe, out in (("pam_migration", pmt.image_file()), ("pam_inversion", pmt.gradient_file())):
        run_single(exe)
        single[exe] = import_bin(out, (pmt.nz, pmt.nx))
        os.remove(out)
    for exe, out in (("pam_migration", pmt.image_file()), ("pam_inversion", pmt.gradient_file())):
        for r in range(2):
            run_rank(exe, r, 2)
        assert not os.path.exists(out)
        red = subprocess.run([os.path.join(BUILD, exe), "--reduce", "2", str(d / "Parameters.json")],
                             capture_output=True, text=True)
        assert red.returncode == 0, red.stdout + red.stderr
        got = import_bin(out, (pmt.nz, pmt.nx))
        err = rel(got, single[exe])
        print(f"{exe}: two ranks + reduce vs one process {err:.2e}")
        assert np.abs(got).max() > 0 and err < 1e-5


def test_driver_reports_missing_model(job, tmp_path):
    d, _ = job
    p = json.loads((d / "Parameters.json").read_text())
    p["vpFile"] = str(tmp_path / "nope.bin")
    p["rec_file"] = str(d / "rec.csv")
    p["src_file"] = str(d / "src.csv")
    (tmp_path / "Parameters.json").write_text(json.dumps(p))
    r = subprocess.run([os.path.join(BUILD, "pam_modeling"), str(tmp_path / "Parameters.json")],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert "Could not open file" in r.stderr


def test_inversion_driver_multiparameter_files(tmp_path):
    """A VTI job with "fwi" and "multiparameter": pam_inversion writes the vp,
    epsilon and delta gradients under the reference's names, and they match
    the reference-shaped Python classes on the same job."""
    from pseudoacousticmodeling_gb300 import build
    from pseudoacousticmodeling_gb300.migration import migration
    from pseudoacousticmodeling_gb300.modeling import wavefield
    from pseudoacousticmodeling_gb300.survey import import_bin, parameters, save_bin, write_csv_geometry
    build.build()
    d = tmp_path
    for sub in ("models", "seis", "img", "grad"):
        (d / sub).mkdir()
    nz, nx, h = 51, 101, 10.0
    vp = np.full((nz, nx), 1600.0, np.float32)
    vp[20:, :] = 2200.0
    eps = np.full((nz, nx), 0.1, np.float32)
    eps[30:, :] = 0.2
    dl = np.full((nz, nx), 0.05, np.float32)
    for name, arr in (("vp", vp), ("eps", eps), ("delta", dl)):
        save_bin(str(d / "models" / f"{name}.bin"), arr)
    write_csv_geometry(d / "rec.csv", np.arange(0, (nx - 1) * h + 1, 2 * h), np.full((nx + 1) // 2, 20.0))
    write_csv_geometry(d / "src.csv", np.array([300.0, 700.0]), np.full(2, 20.0))
    p = {"unit": "GPU", "approximation": "VTI", "migration": "checkpoint", "ABC": "cerjan",
         "dx": h, "dz": h, "dt": 0.001, "L": (nx - 1) * h, "D": (nz - 1) * h, "T": 0.35, "N_abc": 20,
         "fcut": 25.0, "sigma": 3.0, "step": 40, "fwi": True, "multiparameter": True,
         "rec_file": "rec.csv", "src_file": "src.csv", "vpFile": "models/vp.bin", "epsilonFile": "models/eps.bin",
         "deltaFile": "models/delta.bin", "seismogramFolder": "seis/", "imageFolder": "img/",
         "gradientsFolder": "grad/", "batch": 2}
    (d / "Parameters.json").write_text(json.dumps(p))
    _run("pam_modeling", d)
    # invert from a perturbed epsilon so that the data misfit is not zero
    save_bin(str(d / "models" / "eps.bin"), eps * 0.8)
    _run("pam_inversion", d)
    pmt = parameters(str(d / "Parameters.json"))
    files = {k: import_bin(pmt.gradient_file(None if k == "vp" else k), (nz, nx)) for k in ("vp", "epsilon", "delta")}
    for k, v in files.items():
        assert np.isfinite(v).all() and np.abs(v).max() > 0, k
    wf = wavefield(pmt)
    wf.loadModels()
    wf.initializeWavefields()
    wf.setModels()
    mg = migration(wf, pmt)
    g_py, _ = mg.SolveBackwardWaveEquation(save=False)
    assert rel(g_py, files["vp"]) < 1e-6
    for k in ("epsilon", "delta"):
        assert rel(mg.multiparameter_gradients[k], files[k]) < 1e-6, k


def test_gpu_model_smoothing_matches_host():
    """pam_smooth_model (GPU) equals the reference's own compiled smoothing
    (cpp/Migration.cu:131-236; tests/golden/golden_host.npz) bit for bit:
    velocity (slowness smoothing, water layer kept) and epsilon, delta, theta
    (value smoothing) with the water mask of the unsmoothed velocity; and the
    oracle on a larger seeded model."""
    import os
    from pseudoacousticmodeling_gb300 import build
    from pseudoacousticmodeling_gb300.engine import smooth_model
    build.build()
    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_host.npz"))
    for c in G["smooth_cases"]:
        name, field, sigma, parameter = str(c).split("|")
        got = smooth_model(G[f"in_{field}"], float(sigma), parameter == "1", water_model=G["in_vp"])
        np.testing.assert_array_equal(got, G[f"out_{name}"], name)
    rng = np.random.default_rng(5)
    vp = np.full((120, 333), 1500.0, np.float32)
    vp[20:, :] = 2000.0 + 900.0 * rng.random((100, 333)).astype(np.float32)
    g = smooth_model(vp, 6.0)
    np.testing.assert_array_equal(g, O.smooth_model_cpp(vp, 6.0))
    assert (g[:20] == 1500.0).all()
    eps = (0.25 * rng.random((120, 333))).astype(np.float32)
    np.testing.assert_array_equal(smooth_model(eps, 9.5, parameter=True, water_model=vp),
                                  O.smooth_model_cpp(eps, 9.5, parameter=True, water_model=vp))


def test_gpu_laplacian_filter_matches_host_restatement():
    """pam_laplacian_filter (src/Viewdata.py:23-41) on the GPU against the
    host restatement (itself held to the oracle on CPU), including the edge
    copies and grids too small to have an interior."""
    from pseudoacousticmodeling_gb300 import preprocess
    from pseudoacousticmodeling_gb300.engine import laplacian_filter_gpu
    rng = np.random.default_rng(8)
    for nz, nx, dz, dx in ((201, 333, 5.0, 5.0), (37, 12, 8.0, 10.0), (3, 3, 1.0, 2.0)):
        img = (rng.standard_normal((nz, nx)) * 1e-3).astype(np.float32)
        host = preprocess.laplacian_filter(img, dz, dx)
        gpu = laplacian_filter_gpu(img, dz, dx)
        err = np.abs(gpu - host).max() / np.abs(host).max()
        print(f"Laplacian filter {nz}x{nx}: max error relative to the largest value {err:.2e}")
        assert err < 1e-6
    tiny = laplacian_filter_gpu(np.ones((2, 5), np.float32), 1.0, 1.0)
    assert np.array_equal(tiny, np.zeros((2, 5), np.float32))
