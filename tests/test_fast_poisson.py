"""Fast Poisson solve of uniform square arrays (sine transforms instead of the sweeps).

For equal R and C and a uniform self-inductance the face-space matrix of a square array is
kappa times the 5-point Dirichlet Laplacian, the case the reference's SquareArray reserves a
sine-transform solve for (josephson_circuit.py:958). CPU: the recognition of that form. GPU:
the solve against scipy's sparse direct solve (relative 1e-11), trajectories against the
supernodal sweeps and against the oracle (1e-9 relative), and the adjoint through it.
"""
import numpy as np
import pytest
import scipy.sparse.linalg

from oracle import rcsj_oracle
from pyjjasim_gb300 import TimeEvolutionProblem, backend
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray


@pytest.mark.parametrize("n,L,C", [(128, 0.0, 0.0), (256, 0.1, 1.0), (64, 0.05, 0.5)])
def test_recognises_uniform_square_arrays(n, L, C):
    c = SquareArray(n, n)
    c.set_inductance(L)
    c.set_capacitance(C)
    A, K = P.face_matrix(c, 0.05)
    mx, my, grid, kappa = P.fast_poisson_grid(c, K)
    assert (mx, my) == (n - 1, n - 1) and sorted(grid.tolist()) == list(range(K.shape[0]))
    np.testing.assert_allclose(kappa, L + 1.0 / (C / 0.05 ** 2 + 1.0 / 0.05), rtol=1e-14)


def test_rejects_other_circuits():
    c = SquareArray(64, 64)
    c.set_resistance(np.random.default_rng(0).uniform(1, 2, c.junction_count()))
    assert P.fast_poisson_grid(c, P.face_matrix(c, 0.05)[1]) is None           # non-uniform R
    c = SquareArray(10, 10)
    assert P.fast_poisson_grid(c, P.face_matrix(c, 0.05)[1]) is None           # 9 + 1 not a power of two
    c = HoneycombArray(8, 8)
    assert P.fast_poisson_grid(c, P.face_matrix(c, 0.05)[1]) is None


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,W", [(64, 64, 1), (128, 128, 3), (32, 64, 2), (256, 256, 1), (1024, 1024, 1)])
def test_fast_poisson_solve_matches_scipy(nx, ny, W):
    c = SquareArray(nx, ny)
    c.set_inductance(0.07)
    c.set_capacitance(0.3)
    A, K = P.face_matrix(c, 0.05)
    b = np.random.default_rng(nx + W).standard_normal((K.shape[0], W))
    x = backend.solve_faces(c, 0.05, b, fast_poisson=True)
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())


@pytest.mark.gpu
@pytest.mark.parametrize("lines", [1, 2])
@pytest.mark.parametrize("nx,ny,W", [(64, 32, 3), (256, 256, 1)])
def test_one_and_two_lines_per_block_agree(nx, ny, W, lines):
    c = SquareArray(nx, ny)
    A, K = P.face_matrix(c, 0.05)
    b = np.random.default_rng(5).standard_normal((K.shape[0], W))
    x = backend.solve_faces(c, 0.05, b, fast_poisson=True, tuning={"dst_lines": lines})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())


def _problem(c, W, Nt):
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.4, 1.6, W)[None, :, None]
    return TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, current_sources=Is, external_flux=0.13,
                                store_time_steps=np.arange(0, Nt, 25))


@pytest.mark.gpu
@pytest.mark.parametrize("W", [1, 4])
def test_trajectory_matches_sweeps_and_oracle(W):
    c = SquareArray(32, 32)
    c.set_capacitance(0.4)
    c.set_inductance(0.1)
    prob = _problem(c, W, 300)
    th_f, I_f = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, fast_poisson=True)
    th_s, I_s = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, fast_poisson=False)
    th_o, I_o = rcsj_oracle.evolve(prob, prob.store_time_steps, prob.store_time_steps)
    scale = max(1.0, float(np.abs(th_o).max()))
    assert float(np.abs(th_f - th_s).max()) <= 1e-10 * scale
    assert float(np.abs(th_f - th_o).max()) <= 1e-9 * scale
    assert float(np.abs(I_f - I_o).max()) <= 1e-9


@pytest.mark.gpu
def test_plan_uses_the_transforms_by_default_for_single_arrays():
    c = SquareArray(64, 64)
    sim = backend.GpuSimulation(_problem(c, 1, 10))
    assert sim.plan.fast_poisson
    sim = backend.GpuSimulation(_problem(SquareArray(10, 10), 1, 10))
    assert not sim.plan.fast_poisson
