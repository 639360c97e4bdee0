"""FWI on top of the engine: a differentiable modelling operator and the
reference's inversion driver (src/Inversion.py) without its file round trips.

``Propagate`` is a torch.autograd.Function: forward models the shots of a
velocity model (d = F(vp)), backward applies the exact discrete adjoint of the
engine's scheme (pam_misfit_gradient with observed data d - grad_d, whose
residual is grad_d).  Any torch loss on the seismograms therefore
differentiates back to vp.

``fwi`` mirrors the reference class: objective_function, calculate_gradient,
two_loop_recursion, step_length and solveFullWaveformInversion, with the model
parameter m = 1/vp^2 (src/Inversion.py:301) and the gradient preconditioned by
the source illumination as the reference does (src/Migration.py:1086).
"""
import os

import numpy as np

from .engine import Engine

try:
    import torch
except ImportError:   # the autograd entry point needs torch; the rest does not
    torch = None


def _as_np(x):
    if torch is not None and isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


if torch is not None:
    class Propagate(torch.autograd.Function):
        """d = F(vp) for a batch of shots; vp is the interior model [nz][nx]."""

        @staticmethod
        def forward(ctx, vp, engine: Engine, sz, sx, ckpt_interval=0, store="f32"):
            vp_np = np.ascontiguousarray(_as_np(vp), np.float32)
            engine.set_models(vp_np)
            d = engine.forward(sz, sx)
            ctx.engine, ctx.sz, ctx.sx = engine, np.asarray(sz), np.asarray(sx)
            ctx.vp = vp_np
            ctx.ckpt = (int(ckpt_interval), store)
            return torch.from_numpy(d).to(vp.device)

        @staticmethod
        def backward(ctx, grad_d):
            e = ctx.engine
            e.set_models(ctx.vp)
            g = np.ascontiguousarray(grad_d.detach().cpu().numpy(), np.float32)
            # the exact adjoint applied to dL/dd itself (pam_adjoint_gradient)
            gvp = e.adjoint_gradient(ctx.sz, ctx.sx, g, ckpt_interval=ctx.ckpt[0], store=ctx.ckpt[1])
            return torch.from_numpy(gvp).to(grad_d.device), None, None, None, None, None


    class L2Misfit(torch.autograd.Function):
        """J(vp) = 0.5 sum (F(vp) - dobs)^2 with its gradient from one adjoint
        run (no seismograms kept between forward and backward)."""

        @staticmethod
        def forward(ctx, vp, engine: Engine, sz, sx, dobs, ckpt_interval=0, store="f32"):
            vp_np = np.ascontiguousarray(_as_np(vp), np.float32)
            engine.set_models(vp_np)
            J, g = engine.misfit_gradient(sz, sx, np.asarray(_as_np(dobs), np.float32),
                                          ckpt_interval=ckpt_interval, store=store)
            ctx.save_for_backward(torch.from_numpy(g).to(vp.device))
            return torch.tensor(J, dtype=torch.float64, device=vp.device)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout.to(g.dtype) * g, None, None, None, None, None, None


def _dot(a, b):
    return float((a * b).sum())


def two_loop_recursion(g, s_store, y_store):
    """L-BFGS two-loop recursion of src/Inversion.py:88-123, for numpy arrays
    or torch tensors (on any device)."""
    q = g.clone() if hasattr(g, "clone") else g.copy()
    m = len(s_store)
    alpha, rho = [0.0] * m, [0.0] * m
    for i in range(m - 1, -1, -1):
        rho[i] = 1.0 / _dot(y_store[i], s_store[i])
        alpha[i] = rho[i] * _dot(s_store[i], q)
        q = q - alpha[i] * y_store[i]
    gamma = _dot(s_store[-1], y_store[-1]) / _dot(y_store[-1], y_store[-1]) if m else 1.0
    r = gamma * q
    for i in range(m):
        beta = rho[i] * _dot(y_store[i], r)
        r = r + s_store[i] * (alpha[i] - beta)
    return r


class fwi:
    """Monoparameter acoustic FWI (src/Inversion.py:290-411) on a batch engine.

    engine: an Engine for the acoustic approximation; sz, sx: source cells;
    dobs: observed data [shots][nt_data][nrec].

    With torch and a GPU (device "cuda", the default when one is present) the
    whole loop stays on the device, without the reference's file round trips
    (src/Inversion.py:285-288): the model, gradients and L-BFGS history are
    float64 CUDA tensors; the observed data stay resident in HBM, so every
    line-search objective is a device modelling call and a device misfit
    reduction (no seismograms return to the host); the gradient call uploads
    the observed data from pinned memory while its forward sweep runs.
    device "cpu" keeps the same loop in numpy on the host.

    Shots are modelled in batches of the engine's max_shots, and the batches'
    misfits, gradients and illuminations are summed in float64.  Under a
    torch.distributed process group each rank keeps its contiguous share of
    the shots (distributed.local_shots) and the sums of the ranks are added
    with one all-reduce per objective and one per gradient, so every rank
    runs the same L-BFGS iterations on the same model (rank 0 writes the
    checkpoint file)."""

    def __init__(self, engine: Engine, sz, sx, dobs, vmin=1500.0, vmax=5000.0, ckpt_interval=0, store="f32",
                 water_velocity=None, device=None):
        from .distributed import local_shots, world_info
        self.e = engine
        self.rank, self.world = world_info()
        # the problem key covers every shot, whichever share this rank keeps
        self._key_digest = self._digest(sz, sx, dobs)
        self._key_shape = np.shape(dobs)
        idx = local_shots(len(np.atleast_1d(sz)))
        self.sz, self.sx = np.asarray(sz, np.int32)[idx], np.asarray(sx, np.int32)[idx]
        dobs = np.asarray(dobs, np.float32)[idx]
        B = int(getattr(getattr(engine, "cfg", None), "max_shots", len(idx)) or len(idx))
        self.batches = [slice(b, min(b + B, len(idx))) for b in range(0, len(idx), B)]
        self.vmin, self.vmax = vmin, vmax
        self.ckpt = (ckpt_interval, store)
        self.water_velocity = water_velocity
        self.history = []
        if device is None:
            device = "cuda" if torch is not None and torch.cuda.is_available() else "cpu"
        self.gpu = device == "cuda"
        if self.gpu:
            self.stream = torch.cuda.Stream()
            with torch.cuda.stream(self.stream):
                host = torch.empty(np.shape(dobs), dtype=torch.float32).pin_memory()
                host.copy_(torch.from_numpy(np.ascontiguousarray(dobs, np.float32)))
                self.dobs = host.numpy()                       # pinned: the upload overlaps the sweep
                self.d_dobs = host.to("cuda", non_blocking=True)
                # one batch of modelled data, reused by every batch (so the
                # engine's cached time-loop graph keeps its output buffer)
                nb = max(b.stop - b.start for b in self.batches)
                self.d_seis = torch.empty((nb,) + tuple(self.d_dobs.shape[1:]), dtype=torch.float32, device="cuda")
                self.d_sz = torch.from_numpy(self.sz).to("cuda")
                self.d_sx = torch.from_numpy(self.sx).to("cuda")
            self.stream.synchronize()
        else:
            self.dobs = np.asarray(dobs, np.float32)

    # -- array helpers: torch float64 on the GPU, numpy float64 on the host
    def _arr(self, a):
        if self.gpu:
            return torch.as_tensor(np.asarray(a, np.float64), device="cuda")
        return np.asarray(a, np.float64)

    def _host(self, a):
        return a.detach().cpu().numpy() if self.gpu else a

    def _clip(self, m):
        lo, hi = 1.0 / self.vmax ** 2, 1.0 / self.vmin ** 2
        return torch.clamp(m, lo, hi) if self.gpu else np.clip(m, lo, hi)

    def _vp32(self, m):
        """Host float32 velocity 1/sqrt(m) of slowness-squared m."""
        vp = 1.0 / (torch.sqrt(m) if self.gpu else np.sqrt(m))
        return self._host(vp).astype(np.float32)

    def _sum_ranks(self, a):
        from .distributed import allreduce_sum
        return allreduce_sum(a) if self.world > 1 else np.asarray(a, np.float64)

    def objective_function(self, m):
        """0.5 sum (dobs - dcal)^2 at slowness-squared model m (src/Inversion.py:13-53)."""
        self.e.set_models(self._vp32(m))
        J = 0.0
        for b in self.batches:
            if self.gpu:
                seis = self.d_seis[:b.stop - b.start]
                self.e.forward_device(self.d_sz[b], self.d_sx[b], seis, stream=self.stream.cuda_stream)
                J += self.e.misfit_device(seis, self.d_dobs[b], stream=self.stream.cuda_stream)
            else:
                d = self.e.forward(self.sz[b], self.sx[b])
                r = self.dobs[b].astype(np.float64) - d
                J += 0.5 * float(np.sum(r * r))
        return float(self._sum_ranks(np.array([J]))[0])

    def calculate_gradient(self, m, precondition=True):
        """Gradient of the misfit with respect to m = 1/vp^2, optionally divided by
        the illumination (src/Migration.py:1086) and zeroed in the water
        (src/Inversion.py:70-72).  Returns (misfit, gradient)."""
        vp32 = self._vp32(m)
        self.e.set_models(vp32)
        n = vp32.size
        acc = np.zeros(1 + 2 * n)               # misfit, gradient, illumination (float64 sums)
        for b in self.batches:
            self.e.rtm_reset()
            J, gvp = self.e.misfit_gradient(self.sz[b], self.sx[b], self.dobs[b], ckpt_interval=self.ckpt[0],
                                            store=self.ckpt[1])
            _, ilum = self.e.fwi_result()       # illumination of the batch just run
            acc[0] += J
            acc[1:1 + n] += np.asarray(gvp, np.float64).ravel()
            acc[1 + n:] += np.asarray(ilum, np.float64).ravel()
        acc = self._sum_ranks(acc)
        J = float(acc[0])
        gvp = acc[1:1 + n].reshape(vp32.shape).astype(np.float32)
        vp = self._arr(vp32)
        gm = self._arr(gvp) * (-0.5 * vp ** 3)        # dvp/dm = -vp^3 / 2
        if precondition:
            ilum = self._arr(acc[1 + n:].reshape(vp32.shape).astype(np.float32))
            gm = gm / (ilum + 1e-5 * ilum.max())
        if self.water_velocity is not None:
            water = (vp - self.water_velocity).abs() < 1e-3 if self.gpu else np.abs(vp - self.water_velocity) < 1e-3
            gm[water] = 0.0
        return J, gm

    def step_length(self, m, p, g, X, alpha0=1.0, c=1e-4, max_tries=10):
        """Armijo backtracking (src/Inversion.py:125-193), model clipped to
        [1/vmax^2, 1/vmin^2] (src/Inversion.py:369-373)."""
        scale = alpha0 * float(abs(m).max()) * 0.01
        gp = _dot(g, p)
        alpha = scale
        for _ in range(max_tries):
            X_new = self.objective_function(self._clip(m + alpha * p))
            if X_new <= X + c * alpha * gp:
                return alpha, X_new
            alpha *= 0.5
        return 0.0, X

    @staticmethod
    def _digest(sz, sx, dobs):
        import hashlib
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(dobs, np.float32).tobytes())
        h.update(np.ascontiguousarray(sz, np.int32).tobytes())
        h.update(np.ascontiguousarray(sx, np.int32).tobytes())
        return h.hexdigest()

    def _problem_key(self, memory):
        """What a saved loop state must match to be resumed by this run: the
        model shape, the shots, a digest of the observed data (of every shot,
        whatever share this rank models), the L-BFGS memory and the velocity
        bounds."""
        return {"key_dobs_sha256": np.array(self._key_digest), "key_dobs_shape": np.array(self._key_shape),
                "key_memory": np.array(int(memory)), "key_bounds": np.array([self.vmin, self.vmax], np.float64)}

    def _check_state(self, st, path, vp0, memory):
        """Raise ValueError when the state in `path` belongs to another problem."""
        key = self._problem_key(memory)
        for name, want in key.items():
            if name not in st.files:
                raise ValueError(f"FWI checkpoint {path} lacks '{name}': it was not written by this version of the "
                                 "loop; remove it to start afresh")
            if not np.array_equal(st[name], want):
                raise ValueError(f"FWI checkpoint {path} belongs to another problem ({name} differs: saved "
                                 f"{st[name]!r}, this run {want!r}); remove it or pass another path")
        shape = tuple(np.shape(vp0))
        if tuple(st["m"].shape) != shape:
            raise ValueError(f"FWI checkpoint {path} holds a {tuple(st['m'].shape)} model, this run starts from "
                             f"{shape}")

    def _save_state(self, path, it, m, g, X, X0, s_store, y_store, memory):
        """The loop state after iteration `it`, written to a temporary file and
        renamed over `path`, so that an interrupted write leaves the previous
        state intact.  It carries the problem key (_problem_key) checked on
        resumption."""
        state = {"iteration": np.array(it), "m": self._host(m), "g": self._host(g), "X": np.array(X),
                 "X0": np.array(X0), "history": np.array(self.history), "pairs": np.array(len(s_store))}
        state.update(self._problem_key(memory))
        for k, (sv, yv) in enumerate(zip(s_store, y_store)):
            state[f"s{k}"] = self._host(sv)
            state[f"y{k}"] = self._host(yv)
        tmp = path + ".tmp.npz"
        np.savez(tmp, **state)
        os.replace(tmp, path)

    def solveFullWaveformInversion(self, vp0, niter=5, memory=8, checkpoint=None):
        """L-BFGS iterations on m = 1/vp^2 starting from vp0; returns the final vp.

        checkpoint: path of an .npz file that holds the loop state (model,
        gradient, misfits, L-BFGS pairs) after every iteration.  If it exists
        when the call starts, the run resumes from it: the iterations it
        records count towards niter, and vp0 only fixes the expected model
        shape.  A state written for another problem (other observed data,
        shots, model shape, L-BFGS memory or velocity bounds) raises
        ValueError instead of being continued.  The reference writes each
        iteration's model and misfit history (src/Inversion.py:353-355,
        399-406) but cannot resume from them."""
        if checkpoint is not None and os.path.exists(checkpoint):
            st = np.load(checkpoint)
            self._check_state(st, checkpoint, vp0, memory)
            it0 = int(st["iteration"])
            m, g = self._arr(st["m"]), self._arr(st["g"])
            X, X0 = float(st["X"]), float(st["X0"])
            self.history = [float(h) for h in st["history"]]
            s_store = [self._arr(st[f"s{k}"]) for k in range(int(st["pairs"]))]
            y_store = [self._arr(st[f"y{k}"]) for k in range(int(st["pairs"]))]
        else:
            it0 = 0
            m = 1.0 / self._arr(vp0) ** 2
            X, g = self.calculate_gradient(m)
            X0 = X
            self.history = [1.0]
            s_store, y_store = [], []
        for it in range(it0, niter):
            p = -two_loop_recursion(g, s_store, y_store)
            p = p / float(abs(p).max())
            alpha, X_new = self.step_length(m, p, g, X)
            if alpha == 0.0:
                break
            m_new = self._clip(m + alpha * p)
            X_new, g_new = self.calculate_gradient(m_new)
            s, y = m_new - m, g_new - g
            if _dot(s, y) > 0:
                s_store.append(s)
                y_store.append(y)
            if len(s_store) > memory:
                s_store.pop(0)
                y_store.pop(0)
            m, g, X = m_new, g_new, X_new
            self.history.append(X / X0)
            if checkpoint is not None and self.rank == 0:
                self._save_state(checkpoint, it + 1, m, g, X, X0, s_store, y_store, memory)
            if checkpoint is not None and self.world > 1:
                import torch.distributed as dist
                dist.barrier()          # every rank resumes from the same file
        return self._vp32(m)


def solve_multiscale(make_engine, sz, sx, observed, freqs, vp0, niter=5, **fwi_args):
    """Frequency continuation of the reference driver (src/Inversion.py:333-411,
    adjustfmax :285-296): for each cutoff frequency in `freqs`, in order, an
    engine built for that frequency (its Ricker, lag and step count follow
    fcut) inverts the observed data of that band, starting from the model the
    previous band ended with.

    make_engine(fcut) -> Engine with models-independent setup done (receivers,
    wavelet); observed(fcut) -> data [shots][nt_data][nrec] of that band.
    Returns (final vp, {fcut: misfit history})."""
    vp = np.asarray(vp0, np.float32)
    histories = {}
    for fc in freqs:
        e = make_engine(fc)
        inv = fwi(e, sz, sx, observed(fc), **fwi_args)
        vp = inv.solveFullWaveformInversion(vp, niter=niter)
        histories[fc] = list(inv.history)
        e.close()
    return vp, histories

