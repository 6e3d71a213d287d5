"""Simulated annealing of junction arrays on the GPU (pyjjasim's AnnealingProblem).

The reference (time_evolution.py:1070-1191) runs ``interval_count`` separate ``compute()`` calls
of ``interval_steps`` steps; after each it rebuilds the vortex configuration of every stored
step on the host, measures the vortex mobility, and multiplies or divides each problem's
temperature by ``T_factor``. Here one ``GpuSimulation`` stays resident for all intervals: the
temperature is a per-problem device array rewritten in place between intervals (the captured
CUDA graphs stay valid), the phases of an interval stay on the device, and the vortex flow
sum_f sum_s |n_{s+1} - n_s| is reduced there (``jja_vortex``); only W numbers per interval go
back to the host. The reference's semantics are kept literally: every interval restarts from
config_at_minus_1 = config_at_minus_2 = the last phase; the mobility divides by
Nf dt (interval_count - 1); five closing runs at T = 0 with half the time step.

The reference ends with a static (Newton) refinement of every problem's final vortex
configuration (``StaticProblem.compute`` of ``get_static_problem(n_p, problem_nr=0)``,
time_evolution.py:1187-1190). ``compute()`` does the same on the GPU, all problems in one
batched Newton iteration (``static.compute_many``), and returns the reference's triple
(status, configurations, temperature profiles); ``run()`` returns the annealed phases, vortex
configurations, temperature profiles and mobilities without it.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .backend import GpuSimulation, _NumpyNoise, _torch
from .problem import TimeEvolutionProblem

__all__ = ["AnnealingProblem", "AnnealingRun"]


@dataclass
class AnnealingRun:
    theta: np.ndarray                  # (Nj, W) phases after the closing T = 0 runs
    vortex_configuration: np.ndarray   # (Nf, W) vortex configuration of those phases
    temperature_profiles: np.ndarray   # (interval_count, W) temperature after each interval's adjustment
    vortex_mobility: np.ndarray        # (interval_count, W) measured mobility of each interval


class _IntervalNoise:
    """The reference's np.random draws, restarted every interval: each compute() call of the
    reference counts its steps from 0 (which matters for the Nj > 500 reuse pattern)."""

    def __init__(self, Nj, W):
        self.Nj, self.W, self.t0, self.gen = Nj, W, 0, _NumpyNoise(Nj, W)

    def restart(self, t0):
        self.t0, self.gen = t0, _NumpyNoise(self.Nj, self.W)

    def __call__(self, i):
        return self.gen(i - self.t0)


class AnnealingProblem:
    """Same constructor and arguments as pyjjasim's AnnealingProblem (time_evolution.py:1115-1128)."""

    def __init__(self, circuit, time_step=0.5, interval_steps=10, external_flux=0.0, current_sources=0,
                 problem_count=1, interval_count=1000, vortex_mobility=0.001, start_T=1.0, T_factor=1.03):
        self.circuit = circuit
        self.time_step = time_step
        self.interval_steps = interval_steps
        self.interval_count = interval_count
        self.vortex_mobility = vortex_mobility
        self.current_sources = current_sources
        self.external_flux = external_flux
        self.problem_count = problem_count
        self.T = start_T * np.ones((1, self.problem_count, 1))
        self.T_factor = T_factor

    def get_vortex_mobility(self, n):
        """Vortex mobility of consecutive vortex configurations n (Nf, W, steps) (:1129-1136)."""
        Nf = self.circuit.face_count()
        return np.sum(np.sum(np.abs(np.diff(n, axis=2)), axis=2), axis=0) / (
            Nf * self.time_step * (self.interval_count - 1))

    def _target(self, iteration):
        v = self.vortex_mobility
        return v[iteration] if np.array(v).size == self.interval_count else \
            v * ((self.interval_count - iteration) / self.interval_count) ** 1.5

    def _problem(self, dt, T):
        f = np.atleast_1d(self.external_flux)[:, None, None]
        return TimeEvolutionProblem(self.circuit, time_step_count=self.interval_steps, time_step=dt,
                                    external_flux=f, current_sources=self.current_sources, temperature=T,
                                    store_current=False, store_voltage=False, stencil_width=3)

    def run(self, noise="philox", seed=None, **options):
        """Anneal on the GPU. ``noise="numpy"`` replays the reference's np.random draws (parity
        with a seeded reference run); the default draws Philox normals on the device."""
        torch = _torch()
        lib = N.lib()
        c = self.circuit
        Nj, Nf, W, L = c._Nj(), c._Nf(), self.problem_count, self.interval_steps
        T = np.array(self.T, dtype=np.float64)
        noise_gen = _IntervalNoise(Nj, W) if noise == "numpy" else noise
        sim = GpuSimulation(self._problem(self.time_step, T), noise=noise_gen, seed=seed, **options)
        Tsrc = sim.srcs["T"]
        dev = sim.dev
        with torch.cuda.device(dev), torch.cuda.stream(sim.stream):
            th_buf = torch.empty((L, Nj, W), dtype=torch.float64, device=dev)
            flow = torch.zeros(W, dtype=torch.int64, device=dev)
            zeros = torch.zeros((Nj, W), dtype=torch.float64, device=dev)
            sim.set_history([zeros, zeros], 0)
            profiles = np.zeros((self.interval_count, W))
            mobility = np.zeros((self.interval_count, W))
            slots = np.arange(L, dtype=np.int64)
            h = ctypes.c_void_p(sim.stream.cuda_stream)
            noisy = (sim.state.noise_mode, sim.noise_gen, sim.per_step_host)
            for i in range(self.interval_count):
                if getattr(Tsrc, "buf", None) is not None:   # a zero start temperature stays zero
                    Tsrc.buf.copy_(torch.from_numpy(np.ascontiguousarray(T[0, :, 0]).reshape(Tsrc.shape)))
                # the reference skips the noise of a call whose temperature is allclose to 0
                # (time_evolution.py:512-519), and then draws nothing from np.random
                if np.allclose(T, 0):
                    sim.state.noise_mode, sim.noise_gen, sim.per_step_host = N.NOISE_NONE, None, False
                else:
                    sim.state.noise_mode, sim.noise_gen, sim.per_step_host = noisy
                if isinstance(noise_gen, _IntervalNoise):
                    noise_gen.restart(sim.state.step)
                last = sim.theta()
                sim.set_history([last, last], sim.state.step)
                sim.run(L, slots, None, th_buf, None, use_graph=True)
                flow.zero_()
                N.check(lib.jja_vortex(sim.plan.handle, ctypes.c_void_p(th_buf.data_ptr()), L, None,
                                       ctypes.c_void_p(flow.data_ptr()), h))
                moved = flow.cpu().numpy().astype(np.float64)     # synchronises the stream
                mob = moved / (Nf * self.time_step * (self.interval_count - 1))
                upper = self._target(i)
                factor = (mob > upper) * (1 / self.T_factor) + (mob <= upper) * self.T_factor
                T = T * factor[..., None]
                profiles[i] = T[0, :, 0]
                mobility[i] = mob
            sim.synchronize()
            theta = sim.theta().clone()
        # five closing runs at T = 0 with half the time step (no noise: the temperature is zero)
        sim0 = GpuSimulation(self._problem(self.time_step / 2, np.zeros((1, W, 1))), **options)
        with torch.cuda.device(dev), torch.cuda.stream(sim0.stream):
            th0 = theta.to(dev)
            for _ in range(5):
                sim0.set_history([th0, th0], sim0.state.step)
                sim0.run(L, use_graph=True)
                th0 = sim0.theta().clone()
            n_out = torch.empty((1, Nf, W), dtype=torch.int32, device=dev)
            N.check(lib.jja_vortex(sim0.plan.handle, ctypes.c_void_p(th0.data_ptr()), 1,
                                   ctypes.c_void_p(n_out.data_ptr()), None, ctypes.c_void_p(sim0.stream.cuda_stream)))
            sim0.synchronize()
        self.T = T
        return AnnealingRun(theta=th0.cpu().numpy(), vortex_configuration=n_out[0].cpu().numpy().astype(int),
                            temperature_profiles=profiles, vortex_mobility=mobility)

    def compute(self, static_solver=None, **run_options):
        """The reference's return value (status, configurations, temperature_profiles)
        (time_evolution.py:1144-1191). The closing static refinement solves every problem's final
        vortex configuration with the sources and flux of problem 0 (the reference passes
        problem_nr=0 for all of them) on the GPU; ``static_solver(circuit, current_sources,
        external_flux, vortex_configuration) -> (configuration, status)`` replaces it."""
        r = self.run(**run_options)
        Nj = self.circuit._Nj()
        Is = np.broadcast_to(np.asarray(self.current_sources, np.float64), (Nj,)) \
            if np.ndim(self.current_sources) <= 1 else np.asarray(self.current_sources)[:, 0, 0]
        f = np.broadcast_to(np.atleast_1d(np.asarray(self.external_flux, np.float64)), (self.circuit._Nf(),))
        if static_solver is not None:
            data = [static_solver(self.circuit, Is, f, r.vortex_configuration[:, p]) for p in range(self.problem_count)]
            return np.array([d[1] for d in data]), [d[0] for d in data], r.temperature_profiles
        from .static import StaticProblem, compute_many
        problems = [StaticProblem(self.circuit, current_sources=Is.copy(), external_flux=f.copy(),
                                  vortex_configuration=r.vortex_configuration[:, p]) for p in range(self.problem_count)]
        data = compute_many(problems)
        return np.array([d[1] for d in data]), [d[0] for d in data], r.temperature_profiles
