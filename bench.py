"""Benchmark of the hot path: batched VTI pseudo-acoustic modelling with CPML.

Workload (one bench step): 128 shots of an 801 x 2001 grid at 10 m (901 x
2101 with the 50-cell CPML), 4000 recorded samples plus the 369-step source
delay, 12 Hz Ricker, 2001 receivers per shot; seeded synthetic models
(six layers 1500-4000 m/s, smooth epsilon in [0, 0.25] and delta in [0, 0.1]).
Metric: Gcell-updates/s = (nz+2N)(nx+2N) * nt * shots / seconds / 1e9.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`value` is measured with models and geometry resident in HBM (device entry
point); `e2e` times the host C-ABI call (models uploaded and seismograms
copied back every step).  The reference arm (--impl reference) times the CPU
restatement of the reference's modelling loop on the host cores, on a bounded
sample of the same workload.  The `ref_cuda*` fields time the reference's own
CUDA kernels (compiled unmodified where its sources are present, run by the
driver-API harness under oracle/) beside the engine on the same GPU: GPU
baselines, outside every timed region of the engine.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic HBM bytes per updated cell and shot of the VTI stepping kernel:
# read U(t), read U(t-1), write U(t+1) (12 B) plus the three model arrays
# kappa, epsilon, delta (12 B) shared by the batch.
VTI_FIELD_BYTES = 12.0
VTI_MODEL_BYTES = 12.0
CPML_STRIP_BYTES = 8.0     # the stepping kernel's read of the two strip terms per strip cell


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu, path=None):
        import tempfile
        self.gpu = gpu
        self.proc = None
        self.path = path or os.path.join(tempfile.gettempdir(), f"pam_clocks_gpu{gpu}_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def host_cpu():
    """The host's CPU model and logical core count, for the CPU-baseline records."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            with open("/proc/cpuinfo") as f:
                for ln in f:
                    if ln.lower().startswith("model name"):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    import platform
    return {"cpu_model": model or platform.machine(), "nproc": os.cpu_count()}


def cpu_baseline(wl, seconds=15.0):
    """FP32 CPU restatement of the reference time loop (the oracle), all host
    threads, one shot of the same grid for as many steps as fit in ~seconds."""
    from oracle import oracle as O
    lib = O.lib()
    threads = lib.og_threads()
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=wl.nt, itlag=wl.itlag,
               fcut=wl.fcut, approx=wl.approximation, abc=wl.boundary)
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta, wl.theta)
    st = O._State(g, m, np.float32)
    st.cur[int(wl.sz[0]), int(wl.sx[0])] = 1.0
    st.step()       # first-touch and warm caches
    steps = 0
    t0 = time.perf_counter()
    while True:
        st.step()
        st.cur, st.fut = st.fut, st.cur
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds or steps >= 20000:
            break
    cells = wl.cells_expanded * steps
    return {"value": cells / el / 1e9, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
            "sample": f"1 shot x {steps} time steps of the {wl.nz + 2 * wl.n_abc}x{wl.nx + 2 * wl.n_abc} grid "
                      f"({wl.approximation}/{wl.boundary}), FP32 oracle, {threads} OpenMP threads, {el:.1f} s",
            **host_cpu()}


def ref_cuda_baseline(local, steps=400, shots=16):
    """The reference's own CUDA kernels (cpp/Modeling.cu compiled unmodified,
    run by the oracle's driver-API harness) beside this engine on the same GPU
    and grid: the batched-VTI grid with Cerjan boundaries (the reference's
    CUDA path has no CPML), `steps` time steps, one shot through the reference
    kernels and `shots` batched shots through the engine's host call."""
    from oracle import oracle as O
    from oracle import ref as R
    if R.cubin_path() is None:
        return {"value": None, "error": "the reference cubin was not built (reference sources absent at build time)"}
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.engine import Config
    from pseudoacousticmodeling_gb300.workloads import batched_vti
    wl = batched_vti(shots=shots)
    itlag = 40
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=steps, itlag=itlag, fcut=wl.fcut,
               approx="VTI", abc="cerjan")
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta)
    w = O.ricker_cpp(steps, g.dt, g.fcut, np.float32(2.0 * np.sqrt(np.pi) / g.fcut), g.dx, g.dz)
    R.forward(g, m, w, wl.sx[:1], wl.sz[:1], wl.rx, wl.rz)             # warm-up (module load)
    ref_ms = []
    for _ in range(3):
        _, ms = R.forward(g, m, w, wl.sx[:1], wl.sz[:1], wl.rx, wl.rz)
        ref_ms.append(ms)
    e = Engine(Config(nz=wl.nz, nx=wl.nx, n_abc=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=steps, itlag=itlag,
                      fcut=wl.fcut, approximation="VTI", boundary="cerjan", max_shots=shots), device=local)
    e.set_models(wl.vp, wl.eps, wl.delta)
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    e.forward(wl.sz, wl.sx)                                             # warm-up: tuning, graph
    eng_ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        e.forward(wl.sz, wl.sx)
        eng_ms.append((time.perf_counter() - t0) * 1e3 / shots)
    e.close()
    cells = g.nz_a * g.nx_a * steps
    ref_best, eng_best = min(ref_ms), min(eng_ms)
    return {"value": cells / ref_best / 1e6, "unit": "Gcell-updates/s", "ms_per_shot": ref_best,
            "engine_value": cells / eng_best / 1e6, "engine_ms_per_shot": eng_best, "ratio": ref_best / eng_best,
            "sample": f"VTI 901x2101 grid, Cerjan, {steps} steps: reference kernels one shot per run (device time "
                      f"of their launches, best of 3), engine {shots} shots per host call incl. seismogram "
                      f"download (best of 3)"}


def ref_cuda_plain(local):
    """The plain single-shot case (201 x 401 at 10 m, two layers, 50-cell
    Cerjan border, 2237 steps): the reference's own CUDA kernels (one shot,
    device time of their launches) against one engine host call (the
    persistent time loop, seismograms copied back), best of 3 each."""
    from oracle import oracle as O
    from oracle import ref as R
    if R.cubin_path() is None:
        return {"value": None, "error": "the reference cubin was not built (reference sources absent at build time)"}
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.workloads import plain_acoustic
    wl = plain_acoustic()
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=wl.nt, itlag=wl.itlag,
               fcut=wl.fcut, approx="acoustic", abc="cerjan")
    m = O.Models.build(g, wl.vp)
    w = O.ricker_cpp(wl.nt, g.dt, g.fcut, np.float32(2.0 * np.sqrt(np.pi) / g.fcut), g.dx, g.dz)
    R.forward(g, m, w, wl.sx[:1], wl.sz[:1], wl.rx, wl.rz)             # warm-up (module load)
    ref_ms = min(R.forward(g, m, w, wl.sx[:1], wl.sz[:1], wl.rx, wl.rz)[1] for _ in range(3))
    e = Engine(wl.config(), device=local)
    e.set_models(wl.vp)
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    e.forward(wl.sz, wl.sx)                                             # warm-up
    eng = []
    for _ in range(3):
        t0 = time.perf_counter()
        e.forward(wl.sz, wl.sx)
        eng.append((time.perf_counter() - t0) * 1e3)
    e.close()
    cells = g.nz_a * g.nx_a * wl.nt
    return {"value": cells / ref_ms / 1e6, "unit": "Gcell-updates/s", "ms_per_shot": ref_ms,
            "engine_value": cells / min(eng) / 1e6, "engine_ms_per_shot": min(eng), "ratio": ref_ms / min(eng),
            "sample": f"plain acoustic {g.nz_a}x{g.nx_a} expanded grid, Cerjan, {wl.nt} steps, one shot: reference "
                      f"kernels (device time of their launches) against one engine host call incl. the seismogram "
                      f"copy, best of 3 each"}


def run_reference(args):
    """Reference arm: the CPU restatement of the reference modelling loop."""
    world, rank, local = _dist()
    if rank != 0:
        return
    from pseudoacousticmodeling_gb300.workloads import batched_vti
    wl = batched_vti()
    from oracle import oracle as O
    lib = O.lib()
    threads = lib.og_threads()
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=wl.nt, itlag=wl.itlag,
               fcut=wl.fcut, approx=wl.approximation, abc=wl.boundary)
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta, wl.theta)
    st = O._State(g, m, np.float32)
    st.cur[int(wl.sz[0]), int(wl.sx[0])] = 1.0
    per_step = 8    # time steps of one shot per bench step (a bounded sample)
    for _ in range(args.warmup):
        for _ in range(per_step):
            st.step(); st.cur, st.fut = st.fut, st.cur
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(per_step):
            st.step(); st.cur, st.fut = st.fut, st.cur
    el = time.perf_counter() - t0
    cells = wl.cells_expanded * per_step * args.steps
    value = cells / el / 1e9
    out = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "nz": wl.nz, "nx": wl.nx, "n_abc": wl.n_abc, "shots": wl.shots,
                   "nt": wl.nt, "dt": wl.dt},
        "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} time steps of one shot per bench step on the full grid; the "
                                   "reference's own CPU path is Numba code (src/utils.py), not installable here, "
                                   "so its C restatement runs", **host_cpu()},
        "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_fp32_peak(n=8192, reps=10):
    """FP32 CUDA-core throughput of this GPU, measured as cuBLAS's FP32 GEMM
    with TF32 disabled (the CUDA-core counterpart of the bf16 GEMM in
    MEASURED_PEAKS.json), and the FP32 ridge point against the measured HBM
    copy bandwidth: kernels whose FLOP per algorithmic byte lie below it are
    HBM-bound in the roofline sense."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False
    dev = torch.device("cuda", 0)
    a = torch.randn(n, n, device=dev, dtype=torch.float32)
    b = torch.randn(n, n, device=dev, dtype=torch.float32)
    c = torch.empty(n, n, device=dev, dtype=torch.float32)
    for _ in range(3):
        torch.matmul(a, b, out=c)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        torch.matmul(a, b, out=c)
    e1.record()
    torch.cuda.synchronize()
    s = e0.elapsed_time(e1) / 1e3
    tflops = 2.0 * n ** 3 * reps / s / 1e12
    hbm, src = measured_peak()
    print(json.dumps({"fp32_gemm_tflops": tflops, "gemm": f"{n}^3 FP32, TF32 off, {reps} reps",
                      "hbm_gbs": hbm, "hbm_source": src, "ridge_flop_per_byte": tflops * 1e12 / (hbm * 1e9)}))


def run_ncu_case(args):
    """Small case for kernel captures: the full grid of the VTI bench (901 x
    2101) or, with --ncu-workload tti, of the TTI leg (1301 x 3101), 16 shots
    (wavefields of 250 - 520 MB each, larger than L2), 24 time steps.  With
    --ncu-workload fwi: one exact-gradient call on the FWI grid (601 x 1801
    expanded), 32 shots (138 MB per field buffer), 543 steps (100 samples),
    checkpoints every 20 steps (a few GB on the device).  With --ncu-workload
    rtm_vti: one VTI migration (Cerjan) on the VTI grid, 16 shots, 24 steps,
    every step stored."""
    import torch
    from pseudoacousticmodeling_gb300 import Engine, build
    from pseudoacousticmodeling_gb300.engine import Config
    build.build()
    if args.ncu_workload == "rtm_vti":
        import dataclasses
        from pseudoacousticmodeling_gb300.workloads import batched_vti
        wl = dataclasses.replace(batched_vti(shots=16, scale=args.scale), boundary="cerjan")
        cfg = Config(nz=wl.nz, nx=wl.nx, n_abc=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=24, itlag=8,
                     fcut=wl.fcut, approximation="VTI", boundary="cerjan", max_shots=16)
        e = Engine(cfg)
        e.set_models(wl.vp, wl.eps, wl.delta)
        e.set_receivers(wl.rz, wl.rx)
        dobs = e.forward(wl.sz, wl.sx)
        e.rtm(wl.sz, wl.sx, dobs, 0, "f32")
        img, _ = e.rtm_result("none")
        torch.cuda.synchronize()
        print(json.dumps({"ncu_case": "done", "workload": "VTI RTM, Cerjan", "shots": 16, "nt": cfg.nt,
                          "finite": bool(np.isfinite(img).all())}))
        return
    if args.ncu_workload == "fwi":
        from pseudoacousticmodeling_gb300.workloads import fwi_acoustic
        wl, vtrue, w = fwi_acoustic(shots=32, scale=args.scale)
        wl.nt_data = 100
        w = np.ascontiguousarray(w[:wl.nt])
        e = Engine(wl.config())
        e.set_wavelet(w)
        e.set_receivers(wl.rz, wl.rx)
        e.set_models(vtrue)
        dobs = e.forward(wl.sz, wl.sx)
        e.set_models(wl.vp)
        J, g = e.misfit_gradient(wl.sz, wl.sx, dobs, 20, "f32")
        torch.cuda.synchronize()
        print(json.dumps({"ncu_case": "done", "workload": wl.name, "shots": wl.shots, "nt": wl.nt,
                          "finite": bool(np.isfinite(g).all())}))
        return
    from pseudoacousticmodeling_gb300.workloads import batched_tti, batched_vti
    shots = min(args.shots, 16)
    wl = (batched_tti if args.ncu_workload == "tti" else batched_vti)(shots=shots, scale=args.scale)
    cfg = Config(nz=wl.nz, nx=wl.nx, n_abc=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=24, itlag=8, fcut=wl.fcut,
                 approximation=wl.approximation, boundary=wl.boundary, max_shots=shots)
    e = Engine(cfg)
    if wl.approximation == "TTI":
        e.set_models(wl.vp, wl.eps, wl.delta, wl.theta)
    else:
        e.set_models(wl.vp, wl.eps, wl.delta)
    e.set_receivers(wl.rz, wl.rx)
    seis = e.forward(wl.sz, wl.sx)
    torch.cuda.synchronize()
    print(json.dumps({"ncu_case": "done", "workload": wl.name, "shots": shots, "nt": cfg.nt, "finite": bool(np.isfinite(seis).all())}))


# per cell-update of one shot: forward sweep 12 + the fused adjoint step with
# the gradient and illumination sums 20, plus 12 for each recomputed step
FWI_FIELD_BYTES = 32.0
FWI_RECOMPUTE_BYTES = 12.0


def fwi_leg(args, local):
    """FWI gradient ms/shot, batched + checkpointed against the plain path.

    Both go through the host C-ABI call (observed data uploaded from pinned
    memory, gradient folded and copied back inside the timed call).  Batched: all shots in one
    engine call, F32 checkpoints every `fwi_ckpt` steps, segments recomputed
    into HBM.  Plain: one shot per call and per kernel launch, every time step
    stored (no recomputation), no CUDA graph."""
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.workloads import fwi_acoustic
    wl, vtrue, w = fwi_acoustic(shots=args.fwi_shots, scale=args.scale)
    free0 = torch.cuda.mem_get_info(local)[0]
    e = Engine(wl.config(), device=local)
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    e.set_models(vtrue)
    # observed data from the true model (untimed), in pinned memory so that
    # their upload overlaps the forward sweep
    dobs = torch.empty((wl.shots, wl.nt_data, wl.rx.shape[-1]), dtype=torch.float32).pin_memory().numpy()
    e.forward(wl.sz, wl.sx, out=dobs)
    e.set_models(wl.vp)
    if args.fwi_ckpt > 0:
        K, recomputed = args.fwi_ckpt, None
    else:
        # the segment buffer sized to the free HBM: the gradient job's other
        # buffers (two receiver fields, modelled and observed data) and a
        # safety margin are kept out of the budget
        free = torch.cuda.mem_get_info(local)[0]
        nrec = wl.rx.shape[-1]
        other = 2 * e.field_bytes() * wl.shots + 2 * wl.shots * wl.nt_data * nrec * 4
        K, recomputed = e.plan_checkpoints(free - other - args.fwi_margin_gb * 1e9, "f32")
    e.misfit_gradient(wl.sz, wl.sx, dobs, K, "f32")    # warm-up: buffers
    e.profile(16)     # CUDA events around every 16th step's kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, g = e.misfit_gradient(wl.sz, wl.sx, dobs, K, "f32")
    batched_s = time.perf_counter() - t0
    prof = e.profile_read()
    e.profile(0)
    hbm_batched = (free0 - torch.cuda.mem_get_info(local)[0]) / 1e9
    e.close()
    del e
    peak, _ = measured_peak()
    cells = wl.cells_expanded
    kernels = {}
    # algorithmic bytes per cell and shot: forward step 12 (U(t), U(t-1) in,
    # U(t+1) out); fused adjoint + gradient 20 (w(t+1), w(t+2), U(t) in, w(t)
    # out, and the gradient and illumination partial sums read and written
    # once per group of four shots)
    for cls, name, b in (("step", "step_kernel<acoustic,Cerjan> (forward and recompute)", 12.0),
                         ("adjoint", "adjgrad_kernel (adjoint step + gradient + illumination)", 20.0)):
        ms, n = prof[cls]
        if n:
            gbs = b * cells * wl.shots / (ms / n * 1e-3) / 1e9
            kernels[cls] = {"kernel": name, "ms_per_launch": ms / n, "sampled_launches": n,
                            "alg_bytes_per_cell_shot": b, "achieved_GBs": gbs, "frac": gbs / peak}

    free0 = torch.cuda.mem_get_info(local)[0]
    e1 = Engine(wl.config(max_shots=1), device=local)
    e1.set_wavelet(w)
    e1.set_receivers(wl.rz, wl.rx)
    e1.set_models(wl.vp)
    e1.misfit_gradient(wl.sz[:1], wl.sx[:1], dobs[:1], 0, "f32")    # warm-up
    torch.cuda.synchronize()
    n = min(args.fwi_plain_shots, wl.shots)
    t0 = time.perf_counter()
    for i in range(n):
        e1.misfit_gradient(wl.sz[i:i + 1], wl.sx[i:i + 1], dobs[i:i + 1], 0, "f32")
    plain_s = time.perf_counter() - t0
    hbm_plain = (free0 - torch.cuda.mem_get_info(local)[0]) / 1e9
    e1.close()
    del e1

    cells = wl.cells_expanded
    batched_ms = batched_s / wl.shots * 1e3
    plain_ms = plain_s / n * 1e3
    return {
        "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "n_abc": wl.n_abc, "nt": wl.nt, "shots": wl.shots,
        "receivers": int(wl.rx.size), "fcut": wl.fcut, "band_hz": [5.0, 10.0],
        "batched_ms_per_shot": batched_ms, "plain_ms_per_shot": plain_ms, "speedup": plain_ms / batched_ms,
        "batched": f"{wl.shots} shots per call, F32 checkpoints every {K} steps, earlier segments recomputed, "
                   f"the last kept from the forward sweep",
        "ckpt_interval": K, "recomputed_steps": recomputed,
        "plain": f"1 shot per call, every step stored, no graph ({n} shots timed)",
        "hbm_gb_batched": hbm_batched, "hbm_gb_plain": hbm_plain, "misfit": J,
        "batched_alg_GBs": (FWI_FIELD_BYTES * wl.nt + FWI_RECOMPUTE_BYTES * (recomputed if recomputed is not None
                                                                             else wl.nt)) * cells * wl.shots
                           / batched_s / 1e9,
        "gradient_finite": bool(np.isfinite(g).all()),
        "kernels": kernels,
    }


def fwi_full_leg(args, local):
    """The acoustic FWI configuration run as stated: 501 x 1701 at 10 m, 64
    shots, 3443 steps, 20 L-BFGS iterations of inversion.fwi from the smoothed
    starting model, once with the checkpoint plan sized to the free HBM (all
    64 shots per gradient call) and once with every time step stored (the
    largest batch whose full storage fits, several calls per gradient).
    Reports wall time, gradient ms per shot, the HBM in use and the misfit
    history of each."""
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.inversion import fwi
    from pseudoacousticmodeling_gb300.workloads import fwi_acoustic
    wl, vtrue, w = fwi_acoustic(shots=args.fwi_shots, scale=args.scale)
    e = Engine(wl.config(), device=local)
    e.set_wavelet(w)
    e.set_receivers(wl.rz, wl.rx)
    e.set_models(vtrue)
    dobs = torch.empty((wl.shots, wl.nt_data, wl.rx.shape[-1]), dtype=torch.float32).pin_memory().numpy()
    e.forward(wl.sz, wl.sx, out=dobs)
    field = e.field_bytes()
    e.close()
    del e
    out = {"leg": "fwi_full", "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "nt": wl.nt, "shots": wl.shots,
           "iterations": args.fwi_iters}
    nrec = wl.rx.shape[-1]
    for name in ("checkpointed", "full_storage"):
        torch.cuda.synchronize()
        free0, total = torch.cuda.mem_get_info(local)
        if name == "checkpointed":
            B = wl.shots
            e = Engine(wl.config(max_shots=B), device=local)
            other = 2 * field * B + 3 * B * wl.nt_data * nrec * 4
            K, rec = e.plan_checkpoints(free0 - other - args.fwi_margin_gb * 1e9, "f32")
        else:
            # every step stored: nt + 2 fields per shot of the batch, plus the
            # job's other fields and data
            per_shot = (wl.nt + 2 + 6) * field + 3 * wl.nt_data * nrec * 4
            B = int(max(1, min(wl.shots, (free0 - args.fwi_margin_gb * 1e9) // per_shot)))
            while wl.shots % B:
                B -= 1
            e = Engine(wl.config(max_shots=B), device=local)
            K, rec = 0, 0
        e.set_wavelet(w)
        e.set_receivers(wl.rz, wl.rx)
        inv = fwi(e, wl.sz, wl.sx, dobs, vmin=1400.0, vmax=4000.0, ckpt_interval=K, store="f32")
        calls = {"grad_s": 0.0, "grad_n": 0, "obj_s": 0.0, "obj_n": 0}
        grad_fn, obj_fn = inv.calculate_gradient, inv.objective_function

        def timed_grad(m, precondition=True):
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = grad_fn(m, precondition)
            torch.cuda.synchronize()
            calls["grad_s"] += time.perf_counter() - t
            calls["grad_n"] += 1
            return r

        def timed_obj(m):
            t = time.perf_counter()
            r = obj_fn(m)
            calls["obj_s"] += time.perf_counter() - t
            calls["obj_n"] += 1
            return r
        inv.calculate_gradient, inv.objective_function = timed_grad, timed_obj
        t0 = time.perf_counter()
        vp = inv.solveFullWaveformInversion(wl.vp, niter=args.fwi_iters)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        free1, _ = torch.cuda.mem_get_info(local)
        err0 = float(np.linalg.norm(wl.vp - vtrue) / np.linalg.norm(vtrue))
        err1 = float(np.linalg.norm(vp - vtrue) / np.linalg.norm(vtrue))
        out[name] = {"batch": B, "ckpt_interval": K, "recomputed_steps": rec, "wall_s": wall,
                     "gradient_calls": calls["grad_n"], "objective_calls": calls["obj_n"],
                     "gradient_ms_per_shot": calls["grad_s"] / max(calls["grad_n"], 1) / wl.shots * 1e3,
                     "objective_ms_per_shot": calls["obj_s"] / max(calls["obj_n"], 1) / wl.shots * 1e3,
                     "hbm_gb_in_use": (total - free1) / 1e9, "misfit_history": [float(h) for h in inv.history],
                     "model_rel_error_start": err0, "model_rel_error_end": err1}
        e.close()
        del e, inv
    return out


def tti_leg(args, local):
    """Batched TTI modelling (1201 x 3001 at 8 m, 64 shots, 6591 steps): the
    graph-captured batched path against the plain per-shot path (one shot per
    call, one launch per kernel, no graph), Gcell-updates/s.

    The border is the reference's TTI border, Cerjan (cpp/Modeling.cu:731-749),
    unless --tti-boundary CPML: the reference has no CPML for TTI, and the
    engine's CPML, which stretches px, pz, pxx, pzz as for VTI and leaves the
    cross derivative unstretched, becomes unstable on this workload after
    2000 - 4000 steps (non-finite seismograms, PAM_E_NUMERIC), while the same
    models are stable with the Cerjan border, with zero tilt, or without
    anisotropy."""
    import dataclasses
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.workloads import batched_tti
    wl = batched_tti(shots=args.tti_shots, scale=args.scale)
    wl = dataclasses.replace(wl, boundary=args.tti_boundary,
                             name=f"batched TTI pseudo-acoustic modelling, {args.tti_boundary}")
    e = Engine(wl.config(), device=local)
    e.set_models(wl.vp, wl.eps, wl.delta, wl.theta)
    e.set_receivers(wl.rz, wl.rx)
    out = torch.empty((wl.shots, wl.nt_data, wl.rx.shape[-1]), dtype=torch.float32).pin_memory().numpy()
    e.forward(wl.sz, wl.sx, out=out)                         # warm-up: tuning, graph
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.forward(wl.sz, wl.sx, out=out)
    batched_s = time.perf_counter() - t0
    e.close()
    del e
    e1 = Engine(wl.config(max_shots=1), device=local)
    e1.set_models(wl.vp, wl.eps, wl.delta, wl.theta)
    e1.set_receivers(wl.rz, wl.rx)
    os.environ["PAM_NO_GRAPH"] = "1"
    try:
        e1.forward(wl.sz[:1], wl.sx[:1])                     # warm-up: tuning
        torch.cuda.synchronize()
        n = min(args.plain_shots, wl.shots)
        t0 = time.perf_counter()
        for i in range(n):
            e1.forward(wl.sz[i:i + 1], wl.sx[i:i + 1], out=out[i:i + 1])
        plain_s = time.perf_counter() - t0
    finally:
        del os.environ["PAM_NO_GRAPH"]
    e1.close()
    cells = wl.cells_expanded * wl.nt
    ref = None
    if args.tti_boundary == "cerjan":
        try:
            ref = ref_cuda_forward(wl, "TTI", batched_s / wl.shots * 1e3)
        except Exception as ex:  # the comparison is optional: its absence must not void the leg
            ref = {"value": None, "error": str(ex)}
    return {"leg": "tti", "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "nt": wl.nt, "shots": wl.shots,
            "metric": "Gcell-updates/s", "batched": cells * wl.shots / batched_s / 1e9,
            "plain": cells * n / plain_s / 1e9, "plain_shots_timed": n,
            "batched_ms_per_shot": batched_s / wl.shots * 1e3, "plain_ms_per_shot": plain_s / n * 1e3,
            "note": "host C-ABI calls; seismograms copied back to pinned memory inside the timed call",
            "ref_cuda": ref}


def ref_cuda_forward(wl, approx, engine_ms_per_shot):
    """The reference's own forward kernels (cpp/Modeling.cu compiled
    unmodified, in its shot loop restated by the driver-API harness) on the
    first shot of the same workload, all its time steps, Cerjan borders:
    device time of the loop (best of 2) beside this engine's batched host
    call per shot."""
    from oracle import oracle as O
    from oracle import ref as R
    if R.cubin_path() is None:
        return {"value": None, "error": "the reference cubin was not built (reference sources absent at build time)"}
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=wl.nt, itlag=wl.itlag, fcut=wl.fcut,
               approx=approx, abc="cerjan")
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta, wl.theta)
    w = O.ricker_cpp(wl.nt, g.dt, g.fcut, np.float32(2.0 * np.sqrt(np.pi) / g.fcut), g.dx, g.dz)
    ms = min(R.forward(g, m, w, wl.sx[:1], wl.sz[:1], wl.rx, wl.rz)[1] for _ in range(2))
    cells = wl.cells_expanded * wl.nt
    return {"value": cells / ms / 1e6, "unit": "Gcell-updates/s", "ms_per_shot": ms,
            "engine_ms_per_shot": engine_ms_per_shot, "ratio": ms / engine_ms_per_shot,
            "sample": f"one shot, {wl.nt} steps, the reference's forward kernels (device time of the loop, best of "
                      f"2) against this engine's {wl.shots}-shot host call per shot (seismograms to pinned memory)"}


def rtm_leg(args, local):
    """Acoustic RTM (1001 x 4001 at 5 m, 8443 steps, split-spread shots with
    1601 receivers each): ms/shot and image error for checkpoints every 100
    steps stored in FP32, BF16 or FP16 (per-snapshot scale)."""
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.engine import laplacian_filter_gpu as laplacian_filter
    from pseudoacousticmodeling_gb300.workloads import rtm_acoustic
    wl, vtrue = rtm_acoustic(shots=args.rtm_shots, scale=args.scale)
    e = Engine(wl.config(), device=local)
    e.set_receivers(wl.rz, wl.rx, per_shot=True)
    e.set_models(vtrue)
    dobs = torch.empty((wl.shots, wl.nt_data, wl.rx.shape[-1]), dtype=torch.float32).pin_memory().numpy()
    e.forward(wl.sz, wl.sx, out=dobs)                        # observed data (untimed, pinned)
    e.set_models(wl.vp)
    out = {"leg": "rtm", "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "nt": wl.nt, "shots": wl.shots,
           "receivers_per_shot": int(wl.rx.shape[1]), "ckpt_interval": args.rtm_ckpt}
    images = {}
    # checkpoints every rtm_ckpt steps in three formats, then boundary saving
    # (the band of every step) in two
    runs = [("f32", args.rtm_ckpt, "f32"), ("bf16", args.rtm_ckpt, "bf16"), ("f16", args.rtm_ckpt, "f16"),
            ("sb_f32", -1, "f32"), ("sb_f16", -1, "f16")]
    for i, (name, K, store) in enumerate(runs):
        if i == 0:
            e.rtm(wl.sz, wl.sx, dobs, K, store)              # warm-up: buffers, tuning
            e.rtm_reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.rtm(wl.sz, wl.sx, dobs, K, store)
        img, _ = e.rtm_result("cpp")
        el = time.perf_counter() - t0
        free, total = torch.cuda.mem_get_info(local)     # this strategy's buffers are now the allocated ones
        raw, _ = e.rtm_result("none")
        e.rtm_reset()
        images[name] = laplacian_filter(raw, wl.dz, wl.dx)
        images[name + "_cpp"] = laplacian_filter(img, wl.dz, wl.dx)
        out[f"{name}_ms_per_shot"] = el / wl.shots * 1e3
        out[f"{name}_hbm_gb_in_use"] = (total - free) / 1e9
    # errors of the cross-correlation image (before normalisation) after the
    # Laplacian filter; the C++ normalisation divides by the illumination
    # wherever it exceeds an absolute 1e-12, which amplifies any perturbation
    # in barely illuminated cells, so its error is reported separately
    ref = images["f32"].astype(np.float64)
    ref_cpp = images["f32_cpp"].astype(np.float64)
    for name in ("bf16", "f16", "sb_f32", "sb_f16"):
        out[f"{name}_image_rel_l2_vs_f32"] = float(np.linalg.norm(images[name] - ref) / np.linalg.norm(ref))
        out[f"{name}_normalised_image_rel_l2_vs_f32"] = float(
            np.linalg.norm(images[name + "_cpp"] - ref_cpp) / np.linalg.norm(ref_cpp))
    out["cells_per_shot_step"] = wl.cells_expanded
    e.close()
    try:
        out["ref_cuda"] = ref_cuda_rtm(wl, "acoustic", wl.rx[0], wl.rz[0], dobs[:1], out["f32_ms_per_shot"])
    except Exception as ex:  # the comparison is optional: its absence must not void the leg
        out["ref_cuda"] = {"value": None, "error": str(ex)}
    return out


def rtm_vti_leg(args, local):
    """VTI RTM on the modelling workload's grid: 801 x 2001 at 10 m with a
    50-cell Cerjan border (the reference's anisotropic migration has Cerjan
    borders only), 4369 steps, `rtm_shots` shots per call, F32 checkpoints
    every `rtm_ckpt` steps.  Each backward step runs the receiver injection,
    the imaging sum and the anisotropic adjoint (one tiled pass, no scratch
    fields).  Reports ms/shot and, from CUDA events on every 16th backward
    step, the adjoint kernel's time per launch against its algorithmic bytes:
    per cell and shot it reads the source field, the receiver field and its
    previous step and writes the new step (16 B); the model arrays (eps,
    delta, kappa) are shared by the batch."""
    import dataclasses
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.workloads import batched_vti
    wl = batched_vti(shots=args.rtm_shots, scale=args.scale)
    wl = dataclasses.replace(wl, boundary="cerjan", name="VTI RTM, Cerjan, modelling grid")
    e = Engine(wl.config(), device=local)
    e.set_receivers(wl.rz, wl.rx)
    e.set_models(wl.vp, wl.eps, wl.delta)
    dobs = torch.empty((wl.shots, wl.nt_data, wl.rx.shape[-1]), dtype=torch.float32).pin_memory().numpy()
    e.forward(wl.sz, wl.sx, out=dobs)                        # observed data (untimed, pinned)
    e.rtm(wl.sz, wl.sx, dobs, args.rtm_ckpt, "f32")          # warm-up: buffers, tuning
    e.rtm_reset()
    e.profile(16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.rtm(wl.sz, wl.sx, dobs, args.rtm_ckpt, "f32")
    img, _ = e.rtm_result("cpp")
    el = time.perf_counter() - t0
    prof = e.profile_read()
    free, total = torch.cuda.mem_get_info(local)
    e.profile(0)
    e.close()
    peak, _ = measured_peak()
    try:
        ref_rtm = ref_cuda_rtm(wl, "VTI", wl.rx, wl.rz, dobs[:1], el / wl.shots * 1e3)
    except Exception as ex:  # the comparison is optional: its absence must not void the leg
        ref_rtm = {"value": None, "error": str(ex)}
    adj_ms, adj_n = prof["adjoint"]
    img_ms, img_n = prof["imaging"]
    step_ms, step_n = prof["step"]
    cells = wl.cells_expanded
    adj_launch = adj_ms / max(adj_n, 1)
    adj_gbs = 16.0 * cells * wl.shots / (adj_launch * 1e-3) / 1e9 if adj_n else None
    return {"leg": "rtm_vti", "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "nt": wl.nt, "shots": wl.shots,
            "ckpt_interval": args.rtm_ckpt, "ms_per_shot": el / wl.shots * 1e3, "hbm_gb_in_use": (total - free) / 1e9,
            "adjoint_kernel": {"name": "aniso_adjoint_tile_kernel<VTI>", "ms_per_launch": adj_launch,
                               "sampled_launches": adj_n, "alg_bytes_per_cell_shot": 16,
                               "achieved_GBs": adj_gbs, "frac": adj_gbs / peak if adj_gbs else None},
            "imaging_ms_per_launch": img_ms / max(img_n, 1),
            "forward_step_ms_per_launch": step_ms / max(step_n, 1),
            "image_finite": bool(np.isfinite(img).all()), "ref_cuda": ref_rtm}


def ref_cuda_rtm(wl, approx, rx, rz, dobs_shot, engine_ms_per_shot):
    """The reference's own on-the-fly migration (cpp/Migration.cu:359-397:
    its forward and migration kernels, compiled unmodified, in the loop the
    driver-API harness restates) of the first shot of the same workload on
    the same GPU, every source field stored (nt fields of the expanded grid):
    device time of its loop (best of 2), beside this engine's checkpointed
    batch.  The reference's own checkpointed form writes its checkpoints to
    disk (cpp/Migration.cu:399-468), so on-the-fly is its fastest form."""
    from oracle import oracle as O
    from oracle import ref as R
    if R.cubin_path() is None or R.migration_cubin_path() is None:
        return {"value": None, "error": "the reference cubins were not built (reference sources absent at build time)"}
    g = O.Grid(nz=wl.nz, nx=wl.nx, N=wl.n_abc, dz=wl.dz, dx=wl.dx, dt=wl.dt, nt=wl.nt, itlag=wl.itlag, fcut=wl.fcut,
               approx=approx, abc="cerjan")
    m = O.Models.build(g, wl.vp, wl.eps, wl.delta)
    w = O.ricker_cpp(wl.nt, g.dt, g.fcut, np.float32(2.0 * np.sqrt(np.pi) / g.fcut), g.dx, g.dz)
    ms = min(R.rtm(g, m, w, wl.sx[:1], wl.sz[:1], rx, rz, dobs_shot)[2] for _ in range(2))
    return {"ms_per_shot": ms, "engine_ms_per_shot": engine_ms_per_shot, "ratio": ms / engine_ms_per_shot,
            "saved_gb": wl.nt * wl.cells_expanded * 4 / 1e9,
            "sample": f"one shot, {wl.nt} steps, the reference's on-the-fly migration kernels (device time of the "
                      f"loop, best of 2) against this engine's {wl.shots}-shot checkpointed call per shot"}


def plain_leg(args, local):
    """Plain acoustic modelling, 201 x 401 with a 50-cell Cerjan border, one
    shot, 2237 steps: one host C-ABI call.  Its fields (0.6 MB) live in L2, so
    a step is bound by latency, not HBM: the leg times the default time loop
    (one persistent cooperative launch per time chunk) and the graph of
    one-step launches (PAM_NO_PERSISTENT), and reports the difference per step
    as the launch overhead the persistent loop removes."""
    import torch
    from pseudoacousticmodeling_gb300 import Engine
    from pseudoacousticmodeling_gb300.workloads import plain_acoustic
    wl = plain_acoustic()
    reps = 5
    times = {}
    for path in ("persistent", "graph"):
        if path == "graph":
            os.environ["PAM_NO_PERSISTENT"] = "1"
        try:
            e = Engine(wl.config(), device=local)
            e.set_models(wl.vp)
            e.set_receivers(wl.rz, wl.rx)
            e.forward(wl.sz, wl.sx)
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(reps):
                t0 = time.perf_counter()
                e.forward(wl.sz, wl.sx)
                best = min(best, time.perf_counter() - t0)
            e.close()
        finally:
            os.environ.pop("PAM_NO_PERSISTENT", None)
        times[path] = best
    cells = wl.cells_expanded * wl.nt
    el = times["persistent"]
    return {"leg": "plain", "workload": wl.name, "nz": wl.nz, "nx": wl.nx, "nt": wl.nt, "metric": "Gcell-updates/s",
            "value": cells / el / 1e9, "ms_per_shot": el * 1e3, "us_per_step": el / wl.nt * 1e6,
            "graph_ms_per_shot": times["graph"] * 1e3, "graph_us_per_step": times["graph"] / wl.nt * 1e6,
            "launch_overhead_us_per_step": (times["graph"] - el) / wl.nt * 1e6,
            "note": "host C-ABI call incl. the seismogram copy, best of 5; fields L2-resident"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--shots", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true",
                    help="skip timing the reference's own CUDA kernels beside the engine")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the grid (testing only)")
    ap.add_argument("--no-fwi", action="store_true", help="skip the FWI gradient leg")
    ap.add_argument("--clocks-csv", default=None,
                    help="where the nvidia-smi samples of the timed region go (default: a temporary file)")
    ap.add_argument("--fwi-shots", type=int, default=64)
    ap.add_argument("--fwi-ckpt", type=int, default=0,
                    help="checkpoint interval of the batched gradient (0: planned from the free HBM)")
    ap.add_argument("--fwi-margin-gb", type=float, default=6.0,
                    help="HBM left out of the checkpoint plan's budget")
    ap.add_argument("--fwi-plain-shots", type=int, default=4)
    ap.add_argument("--workload", default="vti", choices=["vti", "tti", "rtm", "rtm_vti", "plain", "fwi", "fwi_full"],
                    help="vti: the headline batched VTI line; tti / rtm / plain / fwi / fwi_full print that "
                         "workload's line")
    ap.add_argument("--fwi-iters", type=int, default=20, help="L-BFGS iterations of the fwi_full leg")
    ap.add_argument("--tti-shots", type=int, default=64)
    ap.add_argument("--tti-boundary", default="cerjan", choices=["cerjan", "CPML"],
                    help="border of the TTI leg (the reference's TTI border is Cerjan)")
    ap.add_argument("--plain-shots", type=int, default=2)
    ap.add_argument("--rtm-shots", type=int, default=16)
    ap.add_argument("--rtm-ckpt", type=int, default=100)
    ap.add_argument("--ncu-case", action="store_true",
                    help="one short untimed forward run of the workload grid (16 shots, 24 steps) for ncu captures")
    ap.add_argument("--ncu-workload", default="vti", choices=["vti", "tti", "fwi", "rtm_vti"], help="grid of the --ncu-case run")
    ap.add_argument("--fp32-peak", action="store_true",
                    help="measure the FP32 CUDA-core throughput (FP32 GEMM, TF32 off) and the FP32 ridge point")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.ncu_case:
        return run_ncu_case(args)
    if args.fp32_peak:
        return run_fp32_peak()
    if args.workload != "vti":
        import torch
        from pseudoacousticmodeling_gb300 import build
        build.build()
        torch.cuda.set_device(0)
        if args.workload == "fwi":
            print(json.dumps(dict(leg="fwi", **fwi_leg(args, 0))))
            return
        if args.workload == "fwi_full":
            print(json.dumps(fwi_full_leg(args, 0)))
            return
        leg = {"tti": tti_leg, "rtm": rtm_leg, "rtm_vti": rtm_vti_leg, "plain": plain_leg}[args.workload]
        print(json.dumps(leg(args, 0)))
        return

    import torch
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from pseudoacousticmodeling_gb300 import Engine, build
    build.build()
    from pseudoacousticmodeling_gb300.workloads import batched_vti
    wl = batched_vti(shots=args.shots, scale=args.scale)
    cfg = wl.config()
    e = Engine(cfg, device=local)
    e.set_models(wl.vp, wl.eps, wl.delta)
    e.set_receivers(wl.rz, wl.rx)
    nrec = wl.rx.size
    d_sz = torch.tensor(wl.sz, dtype=torch.int32, device="cuda")
    d_sx = torch.tensor(wl.sx, dtype=torch.int32, device="cuda")
    d_seis = torch.empty((wl.shots, cfg.nt_data, nrec), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    # a stream of its own: the engine launches on it and the timing events are
    # recorded on it (a null handle would select the engine's internal stream)
    stream = torch.cuda.Stream()
    e.profile(16)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- warm-up (graph capture happens on the first call)
    for _ in range(max(args.warmup, 3)):
        e.forward_device(d_sz, d_sx, d_seis, stream=stream.cuda_stream)
    torch.cuda.synchronize()

    # ---- timed region: models and geometry resident in HBM; the K steps are
    # enqueued back to back on `stream` between the two events
    barrier()
    torch.cuda.synchronize()
    with Clocks(local, args.clocks_csv) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            e.forward_device(d_sz, d_sx, d_seis, stream=stream.cuda_stream)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    # sampled kernel times of the last step (every 16th time step)
    prof = e.profile_read()
    step_ms, step_cnt = prof["step"]
    cpml_ms, cpml_cnt = prof["cpml"]
    elapsed = ev0.elapsed_time(ev1) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    cells_per_step = wl.cells_expanded * cfg.nt * wl.shots
    value = cells_per_step * args.steps * world / elapsed / 1e9
    clocks = clk.summary()

    # ---- end to end through the host C-ABI call: upload models, model, copy back
    host_seis = torch.empty((wl.shots, cfg.nt_data, nrec), dtype=torch.float32).pin_memory()
    hs = host_seis.numpy()
    e.forward(wl.sz, wl.sx, out=hs, stream=stream.cuda_stream)    # warm the host path (buffers, graph)
    e2e_steps = max(1, min(args.steps, 2))
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    calls = []
    for _ in range(e2e_steps):
        c0 = time.perf_counter()
        e.set_models(wl.vp, wl.eps, wl.delta)
        c1 = time.perf_counter()
        e.forward(wl.sz, wl.sx, out=hs, stream=stream.cuda_stream)
        calls.append((c1 - c0, time.perf_counter() - c1))
    e2e_el = time.perf_counter() - t0
    h2d = 3 * wl.vp.nbytes + wl.sz.nbytes + wl.sx.nbytes
    d2h = hs.nbytes
    e2e = {"value": cells_per_step * e2e_steps * world / e2e_el / 1e9, "unit": "Gcell-updates/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "calls_s": [[round(a, 4), round(b, 4)] for a, b in calls]}

    # ---- roofline of the stepping kernel
    nza, nxa = cfg.nz_abc, cfg.nx_abc
    upd = (nza - 8) * (nxa - 8)
    strip = 2 * (wl.n_abc - 4) * (nza - 8) + 2 * (wl.n_abc - 4) * (nxa - 8)
    alg_bytes = upd * wl.shots * (VTI_FIELD_BYTES + VTI_MODEL_BYTES / wl.shots) + strip * wl.shots * CPML_STRIP_BYTES
    avg_step_s = step_ms / max(step_cnt, 1) / 1e3
    peak, peak_src = measured_peak()
    achieved = alg_bytes / avg_step_s / 1e9 if step_cnt else None
    # the whole time step (every kernel of the step graph): algorithmic bytes
    # of one step over the per-step time of the timed region
    step_time_s = elapsed / (args.steps * cfg.nt)
    whole = alg_bytes / step_time_s / 1e9
    launches = args.steps * (cfg.nt * (1 + (2 if cfg.boundary == "CPML" else 0)) + cfg.nt_data + 1)

    out = {
        "metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded models with the configuration's shapes and ranges)",
        "config": {"workload": wl.name, "nz": wl.nz, "nx": wl.nx, "n_abc": wl.n_abc, "shots_per_gpu": wl.shots,
                   "nt": cfg.nt, "itlag": cfg.itlag, "nt_data": cfg.nt_data, "dt": wl.dt, "dx": wl.dx,
                   "receivers": int(nrec), "fcut": wl.fcut,
                   "l2": "inputs larger than L2 (2 GB of wavefields per step)",
                   "graph": "whole time loop captured in one CUDA graph"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None,
                     "kernel": "step_kernel<VTI,CPML>", "peak_source": peak_src,
                     "avg_launch_ms": avg_step_s * 1e3, "sampled_launches": step_cnt,
                     "alg_bytes_per_launch": alg_bytes,
                     "whole_step": {"achieved": whole, "frac": whole / peak, "ms_per_time_step": step_time_s * 1e3,
                                    "what": "algorithmic bytes of one time step over the time step's share of the "
                                            "timed region (every kernel of the step graph)"}},
        "interior": {"value": value * wl.nz * wl.nx / wl.cells_expanded, "unit": "Gcell-updates/s",
                     "what": f"the same time over the {wl.nz}x{wl.nx} interior cells only (value counts the "
                             f"{wl.nz + 2 * wl.n_abc}x{wl.nx + 2 * wl.n_abc} expanded grid)"},
        "kernel_share": {"step_ms_sampled": step_ms, "cpml_ms_sampled": cpml_ms,
                         "cpml_over_step": (cpml_ms / step_ms) if step_ms else None},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if not args.no_fwi:
        e.close()
        del e
        fwi = fwi_leg(args, local)
        if world > 1:
            for key in ("batched_ms_per_shot", "plain_ms_per_shot"):
                t = torch.tensor([fwi[key]], device="cuda")
                torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
                fwi[key] = float(t.item())
            fwi["speedup"] = fwi["plain_ms_per_shot"] / fwi["batched_ms_per_shot"]
        out["fwi_gradient"] = fwi
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            out["cpu_baseline"] = cpu_baseline(wl)
        except Exception as ex:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "error": str(ex)}
    if rank == 0 and world == 1 and not args.no_ref_cuda:
        try:
            out["ref_cuda"] = ref_cuda_baseline(local)
        except Exception as ex:  # the baseline is reported, never required
            out["ref_cuda"] = {"value": None, "error": str(ex)}
        try:
            out["ref_cuda_plain"] = ref_cuda_plain(local)
        except Exception as ex:
            out["ref_cuda_plain"] = {"value": None, "error": str(ex)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
