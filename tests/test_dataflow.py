"""Dataflow schedule of the triangular solves (one persistent launch per sweep, work items
waiting on per-supernode completion counters) against scipy's sparse direct solve and against
the level-synchronous schedule, for both fill-reducing orderings and several batch widths."""
import numpy as np
import pytest
import scipy.sparse.linalg

from pyjjasim_gb300 import TimeEvolutionProblem, backend
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray

pytestmark = pytest.mark.gpu


def _solve(circuit, dt, b, ordering, tuning):
    import torch
    W = b.shape[1]
    pl = P.get_plan(circuit, dt, W, 3, ((1.0, -1.0, 0.0), (1.0, -2.0, 1.0)), ordering=ordering, tuning=tuning)
    bd = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    xd = torch.empty_like(bd)
    torch.cuda.synchronize()
    pl.solve(bd.data_ptr(), xd.data_ptr())
    pl.check()
    return xd.cpu().numpy()


@pytest.mark.parametrize("make,W", [(lambda: SquareArray(9, 13), 1), (lambda: SquareArray(30, 30), 37),
                                    (lambda: HoneycombArray(6, 5), 64), (lambda: TriangularArray(7, 6), 3),
                                    (lambda: SquareArray(64, 64), 8)])
@pytest.mark.parametrize("ordering", ["nd", "mmd"])
@pytest.mark.parametrize("rpl", [2, 4, 8])
def test_dataflow_solve_matches_scipy(make, W, ordering, rpl):
    c = make()
    c.set_inductance(0.05)
    dt = 0.05
    A, K = P.face_matrix(c, dt)
    b = np.random.default_rng(W + rpl).standard_normal((K.shape[0], W))
    x = _solve(c, dt, b, ordering, {"schedule": 2, "rows_per_lane": rpl})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    scale = max(1.0, float(np.abs(ref).max()))
    assert float(np.abs(x - ref).max()) <= 1e-11 * scale


@pytest.mark.parametrize("ordering", ["nd", "mmd"])
def test_dataflow_trajectory_matches_levels(ordering):
    c = SquareArray(40, 33)
    c.set_capacitance(0.5)
    W = 24
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.2, 1.9, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=300, current_sources=Is, external_flux=0.15,
                                store_time_steps=[99, 299])
    th1, I1 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, ordering=ordering,
                                          tuning={"schedule": 1})
    th2, I2 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, ordering=ordering,
                                          tuning={"schedule": 2})
    scale = max(1.0, float(np.abs(th1).max()))
    assert float(np.abs(th2 - th1).max()) <= 1e-10 * scale
    assert float(np.abs(I2 - I1).max()) <= 1e-9


def test_bounded_wait_reports_and_recovers():
    """A dataflow sweep whose wait counts can never be reached gives up after its bound: the
    call returns, the plan reports the failure once, and the same plan then solves correctly."""
    import time
    from pyjjasim_gb300 import _native as N
    c = SquareArray(40, 40)
    dt = 0.05
    A, K = P.face_matrix(c, dt)
    W = 4
    pl = P.get_plan(c, dt, W, 3, ((1.0, -1.0, 0.0), (1.0, -2.0, 1.0)), tuning={"schedule": 2})
    t0 = time.perf_counter()
    N.check(N.lib().jja_plan_test_wait_limit(pl.handle, None))
    elapsed = time.perf_counter() - t0
    with pytest.raises(N.JJAError, match="ran out of its bound"):
        pl.check()
    pl.check()      # the flag was cleared by the report
    assert elapsed < 30.0
    b = np.random.default_rng(0).standard_normal((K.shape[0], W))
    x = _solve(c, dt, b, "nd", {"schedule": 2})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    assert float(np.abs(x - ref).max()) <= 1e-11 * max(1.0, float(np.abs(ref).max()))


# ---- cooperative schedule: one launch per sweep, levels separated by grid-wide barriers ------
@pytest.mark.parametrize("make,W", [(lambda: SquareArray(9, 13), 1), (lambda: SquareArray(60, 47), 1),
                                    (lambda: HoneycombArray(25, 21), 1), (lambda: TriangularArray(33, 40), 1),
                                    (lambda: SquareArray(30, 30), 37), (lambda: SquareArray(64, 64), 8)])
@pytest.mark.parametrize("ordering", ["nd", "mmd"])
@pytest.mark.parametrize("extra", [{}, {"pack_min_warps": 1}, {"coop_blocks": 3}])
def test_cooperative_solve_matches_scipy(make, W, ordering, extra):
    c = make()
    c.set_inductance(0.05)
    dt = 0.05
    A, K = P.face_matrix(c, dt)
    b = np.random.default_rng(W + len(extra)).standard_normal((K.shape[0], W))
    x = _solve(c, dt, b, ordering, dict(extra, schedule=3))
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    scale = max(1.0, float(np.abs(ref).max()))
    assert float(np.abs(x - ref).max()) <= 1e-11 * scale


@pytest.mark.parametrize("W", [1, 24])
def test_cooperative_trajectory_matches_levels(W):
    """Graph-replayed steps with stored outputs, noise-free: the cooperative sweeps give the
    level-synchronous trajectory."""
    c = SquareArray(40, 33)
    c.set_capacitance(0.5)
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.2, 1.9, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=300, current_sources=Is, external_flux=0.15,
                                store_time_steps=[99, 299])
    th1, I1 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, tuning={"schedule": 1})
    th3, I3 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, tuning={"schedule": 3})
    scale = max(1.0, float(np.abs(th1).max()))
    assert float(np.abs(th3 - th1).max()) <= 1e-10 * scale
    assert float(np.abs(I3 - I1).max()) <= 1e-9


def test_bounded_barrier_reports_and_recovers():
    """A cooperative sweep whose grid barriers can never complete gives up after their bound: the
    call returns, the plan reports it once, and the same plan then solves correctly."""
    import time
    from pyjjasim_gb300 import _native as N
    c = SquareArray(40, 40)
    dt = 0.05
    A, K = P.face_matrix(c, dt)
    pl = P.get_plan(c, dt, 1, 3, ((1.0, -1.0, 0.0), (1.0, -2.0, 1.0)), tuning={"schedule": 3})
    t0 = time.perf_counter()
    N.check(N.lib().jja_plan_test_wait_limit(pl.handle, None))
    elapsed = time.perf_counter() - t0
    with pytest.raises(N.JJAError, match="ran out of its bound"):
        pl.check()
    pl.check()
    assert elapsed < 60.0
    b = np.random.default_rng(1).standard_normal((K.shape[0], 1))
    x = _solve(c, dt, b, "nd", {"schedule": 3})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    assert float(np.abs(x - ref).max()) <= 1e-11 * max(1.0, float(np.abs(ref).max()))
