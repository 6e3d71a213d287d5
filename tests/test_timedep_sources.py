"""Time-dependent sources held on the device in windows of steps, against the CPU oracle.

The reference evaluates time-dependent inputs (arrays with a time axis, or callables of the
step) once per step (time_evolution.py:334-340, 523-531). The GPU path uploads windows of K
steps and indexes them by the on-device step counter; these tests shrink K so that runs cross
many windows, with and without CUDA-graph replays inside a window, and compare with the
oracle at the trajectory bar (1e-9 relative).
"""
import numpy as np
import pytest

from oracle import rcsj_oracle
from pyjjasim_gb300 import TimeEvolutionProblem, backend
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray

pytestmark = pytest.mark.gpu
NT = 250


def close(actual, desired, rtol=1e-9):
    scale = max(1.0, float(np.abs(desired).max()))
    err = float(np.abs(actual - desired).max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:.1e} * {scale:.3e}"


def _array_problem(c, W):
    rng = np.random.default_rng(7)
    Nj, Nf = c.junction_count(), c.face_count()
    t = np.arange(NT) * 0.05
    Is = c.current_base(0.0)[:, None, None] * (0.8 + 0.3 * np.sin(2 * np.pi * 0.05 * t))[None, None, :] \
        * np.linspace(0.5, 1.5, W)[None, :, None]
    f = 0.1 + 0.05 * rng.standard_normal((Nf, 1, 1)) * np.cos(0.3 * t)[None, None, :]
    Vs = np.zeros((Nj, 1, NT))
    Vs[3, 0, :] = 0.02 * np.sin(0.1 * t)
    return TimeEvolutionProblem(c, time_step=0.05, time_step_count=NT, current_sources=Is, external_flux=f,
                                voltage_sources=Vs, store_time_steps=np.arange(0, NT, 5))


@pytest.mark.parametrize("K", [7, 100, None])
def test_windowed_array_sources_match_oracle(K, monkeypatch):
    c = SquareArray(8, 9)
    c.set_capacitance(0.4)
    c.set_inductance(0.3)
    W = 3
    if K is not None:   # window length K for the largest source, the (Nj, W) current
        monkeypatch.setattr(backend, "_WINDOW_BYTES", K * 8 * c.junction_count() * W)
    prob = _array_problem(c, W)
    th_o, I_o, V_o = rcsj_oracle.time_evolution(prob)
    res = prob.compute()
    close(res.get_theta(), th_o)
    close(res.get_current(), I_o)
    close(res.get_voltage(), V_o, rtol=1e-8)


def test_callable_sources_match_oracle(monkeypatch):
    """AC bias and a drifting flux given as callables of the step (the shape of an AC-driven
    run); windows of 40 steps, so graph replays run inside windows."""
    c = HoneycombArray(5, 4)
    c.set_capacitance(1.0)
    W = 2
    base = c.current_base(0.0)
    Nj, Nf = c.junction_count(), c.face_count()
    monkeypatch.setattr(backend, "_WINDOW_BYTES", 40 * 8 * Nj * W)

    def Is(i):
        return base[:, None] * (0.8 + 0.3 * np.sin(2 * np.pi * 0.05 * i * 0.05)) * np.array([1.0, 1.3])[None, :]

    def f(i):
        return np.full((Nf, 1), 0.1 + 1e-4 * i)

    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=NT, current_sources=Is, external_flux=f,
                                store_time_steps=np.arange(3, NT, 11))
    th_o, I_o, V_o = rcsj_oracle.time_evolution(prob)
    res = prob.compute()
    close(res.get_theta(), th_o)
    close(res.get_current(), I_o)
    close(res.get_voltage(), V_o, rtol=1e-8)


def test_window_bounds_are_checked():
    """The library refuses a call whose steps leave the source window (no out-of-range read)."""
    import ctypes
    from pyjjasim_gb300 import _native as N
    c = SquareArray(4, 4)
    prob = _array_problem(c, 2)
    sim = backend.GpuSimulation(prob)
    sim._enter_window(0)
    st = sim.state
    st.src_steps = 10
    with pytest.raises(N.JJAError, match="outside the source window"):
        N.check(N.lib().jja_run(sim.plan.handle, ctypes.byref(st), 11, None, None, 0,
                                ctypes.c_void_p(sim.stream.cuda_stream)))
