"""AnnealingProblem: the oracle's restatement against the reference's own run (golden fixture),
and the GPU annealer against the oracle with the reference's noise draws replayed."""
import numpy as np
import pytest

import golden_cases as gc
from oracle import rcsj_oracle
from pyjjasim_gb300.problem import TimeEvolutionProblem

PARAMS = ("time_step", "interval_steps", "interval_count", "problem_count", "external_flux", "vortex_mobility",
          "start_T", "T_factor")


def _fixture():
    z = gc.load("a1_square6x5_anneal")
    params = {k: z["param_" + k].item() for k in PARAMS}
    return z, gc.circuit(z), params


def test_oracle_annealing_matches_reference():
    z, c, params = _fixture()
    np.random.seed(int(z["seed"]))
    th, n, profiles, mobility = rcsj_oracle.anneal(TimeEvolutionProblem, c, **params)
    np.testing.assert_allclose(profiles, z["temperature_profiles"], rtol=1e-13, atol=0)
    assert np.array_equal(n, z["final_vortex"])
    assert not np.allclose(profiles[:, 0], profiles[:, 1])     # the problems' temperatures diverge


@pytest.mark.gpu
def test_gpu_annealing_matches_oracle():
    from pyjjasim_gb300.annealing import AnnealingProblem
    z, c, params = _fixture()
    np.random.seed(int(z["seed"]))
    run = AnnealingProblem(c, **params).run(noise="numpy")
    np.testing.assert_allclose(run.temperature_profiles, z["temperature_profiles"], rtol=1e-13, atol=0)
    assert np.array_equal(run.vortex_configuration, z["final_vortex"])
    np.random.seed(int(z["seed"]))
    th_o, n_o, prof_o, mob_o = rcsj_oracle.anneal(TimeEvolutionProblem, c, **params)
    np.testing.assert_allclose(run.vortex_mobility, mob_o, rtol=1e-13, atol=0)
    scale = max(1.0, float(np.abs(th_o).max()))
    assert float(np.abs(run.theta - th_o).max()) <= 1e-9 * scale


@pytest.mark.gpu
def test_gpu_annealing_philox_runs_and_cools():
    from pyjjasim_gb300.annealing import AnnealingProblem
    from pyjjasim_gb300.circuit import SquareArray
    c = SquareArray(24, 24)
    run = AnnealingProblem(c, time_step=0.5, interval_steps=10, interval_count=200, problem_count=16,
                           external_flux=0.3, vortex_mobility=0.02, start_T=1.0, T_factor=1.05).run(seed=4)
    assert run.theta.shape == (c.junction_count(), 16) and np.isfinite(run.theta).all()
    assert run.temperature_profiles.shape == (200, 16)
    assert np.all(run.temperature_profiles[-1] < 1.0)          # the target mobility goes to 0: it cools
    # the vortex configuration of the final state is the one its phases give
    n = rcsj_oracle.vortex_configuration(c.get_cycle_matrix(), run.theta[:, :, None])[:, :, 0]
    assert np.array_equal(n, run.vortex_configuration)
