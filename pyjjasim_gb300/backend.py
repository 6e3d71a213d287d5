"""GPU replacement of the reference's time-stepping core.

``time_evolution_core(problem, th_store_mask, I_store_mask)`` has the signature, inputs
and outputs of pyjjasim's ``time_evolution_core`` (time_evolution.py:461-582): it reads
the problem through the same accessors, and returns (th_out, I_out) as float64 arrays of
shape (Nj, W, sum(mask) + stencil_width - 1) whose first stencil_width-1 slots hold the
initial conditions (theta and cp(theta)), followed by the stored steps in order.

The per-step work runs in libjja_gb300 on the GPU; this module only stages inputs, keeps
device buffers (torch tensors, used as device memory) and copies results back. There is no
CPU path: without a CUDA device or the built library the call raises.

Noise. ``noise="numpy"`` consumes the global ``np.random`` state in the reference's call
order (a fresh ``randn(Nj, W)`` per step, or for Nj > 500 one every third step with
permuted rows in between, time_evolution.py:533-538), uploads each draw, and reproduces the
reference's noisy trajectories. ``noise="philox"`` (default) draws fresh normals per
junction, problem and step on the device (Philox4x32-10); its seed defaults to one 63-bit
draw from ``np.random`` so ``np.random.seed`` still makes runs reproducible.
"""
import ctypes

import numpy as np

from . import _native as N
from . import plan as P

_MAX_OUT_BYTES = 8 << 30   # device bytes for stored steps per segment
# bytes the last time_evolution_core call copied host -> device (phase history, sources, noise)
# and device -> host (stored steps), for transfer accounting
last_transfer = {"h2d_bytes": 0, "d2h_bytes": 0}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyjjasim_gb300 needs a CUDA GPU (GB300, sm_103a); none is available")
    return torch


def _is_default_cpr(cpr):
    return type(cpr).__name__ == "DefaultCPR"


def _compact(v):
    """The non-broadcast part of a 2-D view: axes with stride 0 shrink to length 1."""
    return v[:1 if v.strides[0] == 0 else v.shape[0], :1 if v.strides[1] == 0 else v.shape[1]]


def _host_f64(a):
    """A C-contiguous, writable float64 array with a's values: a itself when it already is one
    (no copy of the large inputs), else a copy (torch.from_numpy needs writable memory)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if a.flags.writeable else a.copy()


def _source_is_zero(timedep, getter, N_rows, W):
    """The reference's zero test ``np.allclose(x, 0)`` for time-independent sources
    (time_evolution.py:512-519), evaluated on the non-broadcast part: |x| <= 1e-8 everywhere
    (NaN and inf are not close to 0)."""
    if timedep:
        return False
    v = _compact(np.broadcast_to(np.asarray(getter(0), dtype=np.float64), (N_rows, W)))
    return bool(np.all(np.abs(v) <= 1e-8))


_WINDOW_BYTES = 256 << 20   # device bytes of one window of a time-dependent source
_WINDOW_MAX_STEPS = 4096


class _Source:
    """A source (Is, f, Vs or T) on the device as a strided ``jja_view``.

    Time-independent: one (rows, cols) array, broadcast axes stored once.
    Time-dependent (an (N, W, Nt) array or a callable of the step, time_evolution.py:334-340):
    windows of K consecutive steps stored time-major (K, rows, cols) that the kernels index
    by the on-device step counter. The host fills a window in pinned memory and uploads it
    asynchronously on the simulation's stream; two window slots alternate, so the host
    evaluates window k+1 while the GPU steps through window k.
    """

    def __init__(self, torch, dev, stream, getter, raw, timedep, N_rows, W, Nt, zero):
        self.getter, self.raw, self.timedep, self.N, self.W, self.Nt = getter, raw, timedep, N_rows, W, Nt
        self.torch, self.dev, self.stream = torch, dev, stream
        self.zero = zero
        self.view = N.View(None, 0, 0, 0)
        self.h2d_bytes = 0
        if zero:
            return
        if not timedep:
            v0 = np.broadcast_to(np.asarray(getter(0), dtype=np.float64), (N_rows, W))
            rows, cols = _compact(v0).shape
            self.shape = (rows, cols)
            self.buf = torch.empty(self.shape, dtype=torch.float64, device=dev)
            self.view = N.View(self.buf.data_ptr(), cols if rows > 1 else 0, 1 if cols > 1 else 0, 0)
            host = _host_f64(v0[:rows, :cols])
            with torch.cuda.stream(stream):
                self.buf.copy_(torch.from_numpy(host))
            self.h2d_bytes += host.nbytes
            return
        if callable(raw) or not isinstance(raw, np.ndarray) or raw.ndim != 3:
            rows, cols = N_rows, W        # a callable may change its shape between steps: keep it full
        else:
            rows, cols = _compact(raw[:, :, 0]).shape
        self.shape = (rows, cols)
        self.K = int(max(1, min(_WINDOW_MAX_STEPS, Nt, _WINDOW_BYTES // (8 * rows * cols))))
        self.slots = [None, None]         # per slot: [window index, device buffer, pinned buffer, event]

    def _fill(self, host, t0, n):
        """Steps [t0, t0 + n) into host[:n] (time-major)."""
        rows, cols = self.shape
        if callable(self.raw) or not isinstance(self.raw, np.ndarray) or self.raw.ndim != 3:
            for k in range(n):
                host[k] = np.broadcast_to(np.asarray(self.getter(t0 + k), np.float64), (self.N, self.W))[:rows, :cols]
        else:
            host[:n] = np.moveaxis(self.raw[:rows, :cols, t0:t0 + n], 2, 0)

    def upload_window(self, wi, K):
        """Fill window wi (steps [wi K, wi K + K) within Nt) and enqueue its upload into slot wi % 2."""
        torch = self.torch
        s = wi % 2
        rows, cols = self.shape
        if self.slots[s] is None:
            self.slots[s] = [-1, torch.empty((K, rows, cols), dtype=torch.float64, device=self.dev),
                             torch.empty((K, rows, cols), dtype=torch.float64, pin_memory=True), None]
        slot = self.slots[s]
        if slot[0] == wi:
            return
        if slot[3] is not None:
            slot[3].synchronize()         # the previous upload from this pinned buffer is done
        t0 = wi * K
        n = min(K, self.Nt - t0)
        self._fill(slot[2].numpy(), t0, n)
        with torch.cuda.stream(self.stream):
            slot[1][:n].copy_(slot[2][:n], non_blocking=True)
            slot[3] = torch.cuda.Event()
            slot[3].record(self.stream)
        slot[0] = wi
        self.h2d_bytes += n * rows * cols * 8

    def use_window(self, wi):
        rows, cols = self.shape
        buf = self.slots[wi % 2][1]
        self.view = N.View(buf.data_ptr(), cols if rows > 1 else 0, 1 if cols > 1 else 0, rows * cols)


class _NumpyNoise:
    """Standard normals in the reference's np.random call order (time_evolution.py:533-538)."""

    def __init__(self, Nj, W):
        self.Nj, self.W, self.prev = Nj, W, None

    def __call__(self, i):
        if self.Nj > 500:
            if i % 3 == 0:
                self.prev = np.random.randn(self.Nj, self.W)
            else:
                self.prev = self.prev[np.random.permutation(self.Nj), :]
        else:
            self.prev = np.random.randn(self.Nj, self.W)
        return self.prev


class HostStage:
    """Everything the GPU core reads from a problem before its first CUDA call.

    Reads the reference's problem interface (time_evolution.py:93-408): the circuit
    (``_Nj/_Nf``, and for the plan ``get_cycle_matrix/_Ic/_R/_C/_L``), ``get_problem_count``,
    ``stencil_width``/``stencil``, ``_dt``/``_Nt``, ``config_at_minus_*`` (the initial phase
    history, newest first), and per source (Is, f, Vs, T) its per-step getter ``_Is(i)``..., its
    raw attribute (array or callable) and ``_*_is_timedep``, with the reference's zero test
    (time_evolution.py:512-519). Works on this package's problem mirror and on the reference's
    own ``TimeEvolutionProblem`` alike; needs no GPU."""

    SOURCES = (("Is", "_Is", "_Is_is_timedep", "current_sources", "Nj"),
               ("f", "_f", "_f_is_timedep", "external_flux", "Nf"),
               ("Vs", "_Vs", "_Vs_is_timedep", "voltage_sources", "Nj"),
               ("T", "_T", "_T_is_timedep", "temperature", "Nj"))

    def __init__(self, problem):
        c = problem.get_circuit()
        if not _is_default_cpr(problem.get_current_phase_relation()):
            raise NotImplementedError("the GPU core evaluates the default current-phase relation Ic*sin(theta) only")
        self.problem, self.circuit = problem, c
        self.Nj, self.Nf, self.W = c._Nj(), c._Nf(), problem.get_problem_count()
        self.width = problem.stencil_width
        self.stencil = problem.stencil
        self.dt, self.Nt = problem._dt(), problem._Nt()
        hist0 = [problem.config_at_minus_1, problem.config_at_minus_2]
        if self.width >= 4:
            hist0.append(problem.config_at_minus_3)
        if self.width >= 5:
            hist0.append(problem.config_at_minus_4)
        shape = (self.Nj, self.W)
        self.hist0 = [_host_f64(h if np.shape(h) == shape else np.broadcast_to(h, shape)) for h in hist0]
        self.hist0_zero = [not np.any(h) for h in self.hist0]
        self.sources = {}
        for name, getter, timedep, attr, rows in self.SOURCES:
            get, td, n = getattr(problem, getter), bool(getattr(problem, timedep)), getattr(self, rows)
            self.sources[name] = dict(getter=get, raw=getattr(problem, attr, None), timedep=td, rows=n,
                                      zero=_source_is_zero(td, get, n, self.W))


class GpuSimulation:
    """Device-resident state of W time-evolution problems of one TimeEvolutionProblem.

    Holds the cached plan, the phase history, theta_s and the sources on the GPU. ``run``
    advances any number of steps (optionally storing steps into device output buffers),
    ``run_timed`` advances with per-stage CUDA-event timing, ``theta`` returns the newest phase.
    """

    def __init__(self, problem, noise="philox", seed=None, device=None, nd_leaf=None, stream=None, ordering="auto",
                 relax=(-1, -1.0), Ic=None, tuning=None, tune=False, fast_poisson="auto"):
        """``Ic``: optional (Nj, W) critical currents per problem, replacing the circuit's
        (problems then differ in Ic but share the face-space matrix, which does not depend on Ic).
        ``tuning``: launch shape of the triangular solves (plan.TUNING_FIELDS); ``tune=True``
        takes ``relax`` and ``tuning`` from the autotuner (timed once per GPU, circuit and W,
        then cached on disk). ``fast_poisson``: sine-transform face solves for uniform square
        arrays (plan.get_plan): "auto", True or False."""
        stage = self.stage = HostStage(problem)       # host reads first: no CUDA call before
        torch = self.torch = _torch()
        c = stage.circuit
        self.problem = problem
        self.Nj, self.Nf, self.W = stage.Nj, stage.Nf, stage.W
        self.width = stage.width
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.h2d_bytes = 0
        with torch.cuda.device(self.dev):
            if tune:
                from .autotune import autotune
                opts = autotune(c, stage.dt, self.W, self.width, nd_leaf=nd_leaf, device=self.dev.index)
                ordering, relax, tuning = opts["ordering"], opts["relax"], opts["tuning"]
            self.ordering = P.resolve_ordering(ordering, self.W, self.Nf)
            self.relax, self.tuning = tuple(relax), dict(tuning or {})
            self.stream = stream if stream is not None else torch.cuda.Stream(device=self.dev)
            self.plan = P.get_plan(c, stage.dt, self.W, self.width, stage.stencil, nd_leaf=nd_leaf,
                                   ordering=self.ordering, relax=relax, Ic_w=Ic, tuning=tuning,
                                   fast_poisson=fast_poisson)
            self.hist0, self.hist0_zero = stage.hist0, stage.hist0_zero
            self.hist = []
            with torch.cuda.stream(self.stream):
                for h, zero in zip(stage.hist0, stage.hist0_zero):
                    if zero:      # the default initial condition: no host->device copy needed
                        self.hist.append(torch.zeros((self.Nj, self.W), dtype=torch.float64, device=self.dev))
                    else:
                        self.hist.append(torch.from_numpy(h).to(self.dev))
                        self.h2d_bytes += h.nbytes
            self.srcs = {}
            self.Nt = stage.Nt
            for name, sp in stage.sources.items():
                self.srcs[name] = _Source(torch, self.dev, self.stream, sp["getter"], sp["raw"], sp["timedep"],
                                          sp["rows"], self.W, self.Nt, sp["zero"])
            # time-dependent sources share one grid of step windows
            self.windowed = [s for s in self.srcs.values() if s.timedep and not s.zero]
            self.window_K = min((s.K for s in self.windowed), default=0)
            self.window = -1
            self.h2d_bytes += sum(s.h2d_bytes for s in self.srcs.values())
            Vs_zero, T_zero = self.srcs["Vs"].zero, self.srcs["T"].zero
            self.theta_s = None if Vs_zero else torch.zeros((self.Nj, self.W), dtype=torch.float64, device=self.dev)
            st = self.state = N.State()
            for k in range(4):
                st.hist[k] = self.hist[k].data_ptr() if k < len(self.hist) else None
            st.theta_s = self.theta_s.data_ptr() if self.theta_s is not None else None
            st.Is, st.f, st.Vs, st.T = (self.srcs[k].view for k in ("Is", "f", "Vs", "T"))
            st.step = 0
            self.noise_gen = None
            self.noise_buf = None
            if T_zero:
                st.noise_mode = N.NOISE_NONE
            elif callable(noise):
                self.noise_gen = noise
            elif noise == "numpy":
                self.noise_gen = _NumpyNoise(self.Nj, self.W)
            elif noise == "philox":
                st.noise_mode = N.NOISE_PHILOX
                st.seed = int(np.random.randint(0, 2 ** 63 - 1, dtype=np.int64)) if seed is None else int(seed)
            else:
                raise ValueError(f"unknown noise mode {noise!r}")
            if self.noise_gen is not None:
                st.noise_mode = N.NOISE_BUFFER
                self.noise_buf = torch.empty((self.Nj, self.W), dtype=torch.float64, device=self.dev)
                st.noise = self.noise_buf.data_ptr()
            self.per_step_host = self.noise_gen is not None

    # ----------------------------------------------------------------------------------------
    def _enter_window(self, step):
        """Make the window holding ``step`` current (uploading it if it is not already there);
        returns the number of steps from ``step`` to the end of the window."""
        if not self.windowed:
            return None
        if step >= self.Nt:
            raise ValueError(f"step {step} is past the time-dependent sources ({self.Nt} steps)")
        K = self.window_K
        wi = step // K
        if wi != self.window:
            for s in self.windowed:
                s.upload_window(wi, K)
                s.use_window(wi)
            st = self.state
            st.Is, st.f, st.Vs, st.T = (self.srcs[k].view for k in ("Is", "f", "Vs", "T"))
            st.src_t0 = wi * K
            st.src_steps = min(K, self.Nt - wi * K)
            self.window = wi
        return self.state.src_t0 + self.state.src_steps - step

    def _prefetch_window(self):
        """Fill and enqueue the window after the current one (host work that overlaps the GPU)."""
        nxt = self.window + 1
        if self.windowed and nxt * self.window_K < self.Nt:
            for s in self.windowed:
                s.upload_window(nxt, self.window_K)

    def run(self, nsteps, th_slot=None, I_slot=None, th_dev=None, I_dev=None, use_graph=True, store_all=False):
        """Advance nsteps steps; step i writes th_dev[th_slot[i]] / I_dev[I_slot[i]] when >= 0,
        or, with ``store_all``, th_dev[i] / I_dev[i] for every step (slots derived on the device,
        so those runs replay CUDA graphs as well)."""
        torch, st = self.torch, self.state
        lib = N.lib()
        if store_all and (th_slot is not None or I_slot is not None):
            raise ValueError("store_all replaces th_slot / I_slot")
        st.store_all = 1 if store_all else 0
        slot_bytes = self.Nj * self.W * 8
        st.th_out = th_dev.data_ptr() if th_dev is not None else None
        st.I_out = I_dev.data_ptr() if I_dev is not None else None
        th_slot = None if th_slot is None else np.ascontiguousarray(th_slot, np.int64)
        I_slot = None if I_slot is None else np.ascontiguousarray(I_slot, np.int64)
        h = ctypes.c_void_p(self.stream.cuda_stream)
        k = 0
        while k < nsteps:
            left = self._enter_window(st.step)
            n = nsteps - k if left is None else min(nsteps - k, left)
            if store_all:     # every call numbers its steps from 0: offset the outputs
                st.th_out = th_dev.data_ptr() + k * slot_bytes if th_dev is not None else None
                st.I_out = I_dev.data_ptr() + k * slot_bytes if I_dev is not None else None
            ts = None if th_slot is None else th_slot[k:k + n]
            Is_ = None if I_slot is None else I_slot[k:k + n]
            if not self.per_step_host:
                N.check(lib.jja_run(self.plan.handle, ctypes.byref(st), int(n), N.ptr(ts, ctypes.c_int64),
                                    N.ptr(Is_, ctypes.c_int64), int(use_graph), h))
                self._prefetch_window()
            else:
                for q in range(n):
                    if store_all:
                        st.th_out = th_dev.data_ptr() + (k + q) * slot_bytes if th_dev is not None else None
                        st.I_out = I_dev.data_ptr() + (k + q) * slot_bytes if I_dev is not None else None
                    with torch.cuda.stream(self.stream):
                        self.noise_buf.copy_(torch.from_numpy(
                            np.array(self.noise_gen(st.step), np.float64, order="C")))
                    N.check(lib.jja_run(self.plan.handle, ctypes.byref(st), 1,
                                        N.ptr(ts[q:q + 1], ctypes.c_int64) if ts is not None else None,
                                        N.ptr(Is_[q:q + 1], ctypes.c_int64) if Is_ is not None else None, 0, h))
            k += n

    def run_timed(self, nsteps):
        """Advance nsteps steps (eager) and return per-stage device milliseconds."""
        if self.per_step_host:
            raise ValueError("run_timed needs on-device noise")
        left = self._enter_window(self.state.step)
        if left is not None and left < nsteps:
            raise ValueError("run_timed: the steps cross a window of the time-dependent sources")
        ms = np.zeros(6)
        N.check(N.lib().jja_run_timed(self.plan.handle, ctypes.byref(self.state), int(nsteps), N.ptr(ms),
                                      ctypes.c_void_p(self.stream.cuda_stream)))
        return dict(zip(("first_junction", "face_rhs", "forward", "backward", "update_junction", "total"),
                        ms.tolist()))

    def history(self):
        """Device tensors of the phase history, newest first (theta(t-1), theta(t-2), ...)."""
        by_ptr = {t.data_ptr(): t for t in self.hist}
        return [by_ptr[self.state.hist[k]] for k in range(self.width - 1)]

    def set_history(self, thetas, step):
        """Restart from a saved history (newest first) at global step index ``step``."""
        for dst, src in zip(self.history(), thetas):
            with self.torch.cuda.stream(self.stream):
                dst.copy_(src)
        self.state.step = int(step)

    def theta_ptr(self):
        return self.state.hist[0]

    def theta(self):
        """Newest phase (Nj, W) as a device tensor view."""
        for t in self.hist:
            if t.data_ptr() == self.state.hist[0]:
                return t
        raise RuntimeError("history buffer not found")

    def synchronize(self):
        """Wait for the simulation's stream and check the plan's device error flag."""
        self.stream.synchronize()
        self.plan.check()


def time_evolution_core(problem, th_store_mask, I_store_mask, noise="philox", seed=None, device=None,
                        use_graph=True, nd_leaf=None, stream=None, ordering="auto", relax=(-1, -1.0), Ic=None,
                        tuning=None, tune=False, sim=None, fast_poisson="auto"):
    """GPU time-stepping core; see the module docstring for the contract.

    ``ordering`` ("nd", "mmd" or "auto": minimum degree when W x Nf >= 2^22 on up to 2^18 faces,
    nested dissection otherwise) and ``relax`` ((max zeros, max fraction) of supernode
    amalgamation; negative = library defaults) select how the face-space matrix is factorised;
    ``tuning`` the solve's launch shape; ``tune=True`` lets the autotuner pick both. ``sim``: a
    GpuSimulation of this problem, already built (its own options apply)."""
    if sim is None:
        sim = GpuSimulation(problem, noise=noise, seed=seed, device=device, nd_leaf=nd_leaf, stream=stream,
                            ordering=ordering, relax=relax, Ic=Ic, tuning=tuning, tune=tune, fast_poisson=fast_poisson)
    elif sim.problem is not problem:
        raise ValueError("time_evolution_core: the simulation belongs to another problem")
    torch = sim.torch
    Nj, W, Nt, width = sim.Nj, sim.W, problem._Nt(), sim.width
    th_store_mask = np.asarray(th_store_mask, bool)
    I_store_mask = np.asarray(I_store_mask, bool)
    n_init = width - 1
    n_th, n_I = int(th_store_mask.sum()), int(I_store_mask.sum())
    # outputs are filled time-major, one contiguous (Nj, W) block per slot, and returned as
    # (Nj, W, slots) views: the shape and values of the reference's arrays without a transpose
    th_buf = np.empty((n_th + n_init, Nj, W))
    I_buf = np.empty((n_I + n_init, Nj, W))
    for lag, (th, zero) in enumerate(zip(sim.hist0, sim.hist0_zero)):   # time_evolution.py:480-502
        th_buf[n_init - 1 - lag] = th
        if zero:
            I_buf[n_init - 1 - lag] = 0.0          # cp(0) = Ic sin 0
        else:
            th = np.broadcast_to(th, (Nj, W))
            I_buf[n_init - 1 - lag] = problem._cp(th) if Ic is None else np.asarray(Ic) * np.sin(th)
    th_idx = np.where(th_store_mask, np.cumsum(th_store_mask) - 1, -1).astype(np.int64)
    I_idx = np.where(I_store_mask, np.cumsum(I_store_mask) - 1, -1).astype(np.int64)
    max_slots = max(1, _MAX_OUT_BYTES // (2 * Nj * W * 8))
    d2h = 0
    noise_h2d = 0
    with torch.cuda.device(sim.dev):
        i0 = 0
        while i0 < Nt:
            # segment [i0, i1) holds at most max_slots stored steps of each kind on the device
            i1, cnt_th, cnt_I = i0, 0, 0
            while i1 < Nt:
                a, b = int(th_store_mask[i1]), int(I_store_mask[i1])
                if cnt_th + a > max_slots or cnt_I + b > max_slots:
                    break
                cnt_th, cnt_I, i1 = cnt_th + a, cnt_I + b, i1 + 1
            base_th, base_I = int(th_store_mask[:i0].sum()), int(I_store_mask[:i0].sum())
            seg_th = np.where(th_idx[i0:i1] >= 0, th_idx[i0:i1] - base_th, -1)
            seg_I = np.where(I_idx[i0:i1] >= 0, I_idx[i0:i1] - base_I, -1)
            th_dev = torch.empty((cnt_th, Nj, W), dtype=torch.float64, device=sim.dev) if cnt_th else None
            I_dev = torch.empty((cnt_I, Nj, W), dtype=torch.float64, device=sim.dev) if cnt_I else None
            sim.run(i1 - i0, seg_th, seg_I, th_dev, I_dev, use_graph=use_graph)
            sim.synchronize()
            if cnt_th:
                torch.from_numpy(th_buf[n_init + base_th:n_init + base_th + cnt_th]).copy_(th_dev)
            if cnt_I:
                torch.from_numpy(I_buf[n_init + base_I:n_init + base_I + cnt_I]).copy_(I_dev)
            d2h += (cnt_th + cnt_I) * Nj * W * 8
            if sim.per_step_host:
                noise_h2d += (i1 - i0) * Nj * W * 8
            del th_dev, I_dev
            i0 = i1
    last_transfer["h2d_bytes"] = sim.h2d_bytes + sum(s.h2d_bytes for s in sim.windowed) + noise_h2d
    last_transfer["d2h_bytes"] = d2h
    return th_buf.transpose(1, 2, 0), I_buf.transpose(1, 2, 0)


def solve_faces(circuit, dt, b, stencil_width=3, nd_leaf=8, ordering="auto", tuning=None, fast_poisson=False):
    """K^{-1} b on the GPU for (Nf, W) right-hand sides (the per-step face-space solve);
    ``ordering``, ``tuning`` and ``fast_poisson`` as for the simulation's plan."""
    from .problem import stencil
    torch = _torch()
    b = np.ascontiguousarray(b, np.float64)
    squeeze = b.ndim == 1
    if squeeze:
        b = b[:, None]
    W = b.shape[1]
    pl = P.get_plan(circuit, dt, W, stencil_width, stencil(stencil_width), nd_leaf=nd_leaf, ordering=ordering,
                    tuning=tuning, fast_poisson=fast_poisson)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        bd = torch.from_numpy(b).cuda()
        xd = torch.empty_like(bd)
    st.synchronize()
    pl.solve(bd.data_ptr(), xd.data_ptr(), st.cuda_stream)
    st.synchronize()
    pl.check()
    x = xd.cpu().numpy()
    return x[:, 0] if squeeze else x
