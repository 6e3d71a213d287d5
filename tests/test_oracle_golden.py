"""Pin the CPU oracle against golden vectors produced by the reference's own compute()."""
import numpy as np
import pytest

import golden_cases as gc
from oracle import rcsj_oracle


@pytest.mark.parametrize("name", gc.case_names())
def test_oracle_matches_reference_golden(name):
    z = gc.load(name)
    prob = gc.problem(z)
    s = gc.seed(z)
    if s is not None:
        np.random.seed(s)
    th, I, V = rcsj_oracle.time_evolution(prob)
    # Same library solve and same operation order as the reference: agreement to round-off.
    np.testing.assert_allclose(th, z["theta"], rtol=0, atol=1e-12 * max(1.0, np.abs(z["theta"]).max()))
    np.testing.assert_allclose(I, z["current"], rtol=0, atol=1e-12 * max(1.0, np.abs(z["current"]).max()))
    np.testing.assert_allclose(V, z["voltage"], rtol=0, atol=1e-11 * max(1.0, np.abs(z["voltage"]).max()))
    A = prob.get_circuit().get_cycle_matrix()
    assert np.array_equal(rcsj_oracle.vortex_configuration(A, th), z["vortex"])
