"""Host logic of the TimeEvolutionProblem / time_evolution / TimeEvolutionResult mirror.

The masks, voltage post-processing and result accessors run on the host; with the CPU
oracle plugged in as the core they must reproduce the reference's golden outputs exactly.
"""
import numpy as np
import pytest

import golden_cases as gc
from oracle import rcsj_oracle
from pyjjasim_gb300 import SquareArray, TimeEvolutionProblem
from pyjjasim_gb300.problem import DataAtTimepointNotStored, ThetaNotStored, time_evolution


@pytest.mark.parametrize("name", gc.case_names())
def test_mirror_postprocessing_matches_reference(name):
    z = gc.load(name)
    prob = gc.problem(z)
    s = gc.seed(z)
    if s is not None:
        np.random.seed(s)
    res = time_evolution(prob, core=rcsj_oracle.evolve)
    tol = lambda a: 1e-12 * max(1.0, np.abs(a).max())
    np.testing.assert_allclose(res.get_theta(), z["theta"], rtol=0, atol=tol(z["theta"]))
    np.testing.assert_allclose(res.get_current(), z["current"], rtol=0, atol=tol(z["current"]))
    np.testing.assert_allclose(res.get_voltage(), z["voltage"], rtol=0, atol=10 * tol(z["voltage"]))
    assert np.array_equal(res.get_vortex_configuration(), z["vortex"])


def test_store_flags_and_selection():
    a = SquareArray(5, 4)
    Is = 0.6 * a.current_base(0.0)[:, None, None]
    for flags in [(True, False, False), (False, True, False), (False, False, True), (True, True, True)]:
        prob = TimeEvolutionProblem(a, time_step_count=30, current_sources=Is, external_flux=0.2,
                                    store_time_steps=[0, 3, 4, 10, 29], store_theta=flags[0], store_voltage=flags[1],
                                    store_current=flags[2])
        res = time_evolution(prob, core=rcsj_oracle.evolve)
        th, I, V = rcsj_oracle.time_evolution(prob)
        for arr, ref in ((res.theta, th), (res.voltage, V), (res.current, I)):
            assert (arr is None) == (ref is None)
            if ref is not None:
                np.testing.assert_array_equal(np.asarray(arr), ref)
    prob = TimeEvolutionProblem(a, time_step_count=10, store_time_steps=[2, 5], store_theta=False,
                                store_voltage=True, store_current=False)
    res = time_evolution(prob, core=rcsj_oracle.evolve)
    with pytest.raises(ThetaNotStored):
        res.get_theta()
    with pytest.raises(DataAtTimepointNotStored):
        res.get_voltage(select_time_points=[3])
    assert res.get_voltage(select_time_points=[5]).shape == (a.junction_count(), 1, 1)


def test_problem_validation():
    a = SquareArray(3, 3)
    with pytest.raises(ValueError):
        TimeEvolutionProblem(a, store_theta=False, store_voltage=False, store_current=False)
    with pytest.raises(ValueError):
        TimeEvolutionProblem(a, time_step_count=5, store_time_steps=np.zeros(5, bool))
    with pytest.raises(ValueError):
        TimeEvolutionProblem(a, stencil_width=6)
    # problem count from the widest source, callables evaluated at step 0
    p = TimeEvolutionProblem(a, current_sources=lambda i: np.zeros((a.junction_count(), 7)), time_step_count=3)
    assert p.get_problem_count() == 7 and p._Is_is_timedep
    with pytest.raises(ValueError):       # the GPU core is the only backend: no CPU fallback
        p.compute(backend="numpy")
