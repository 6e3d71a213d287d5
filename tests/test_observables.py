"""Derived observables of a time-evolution result (pyjjasim time_evolution.py:692-985): node
phases and potentials, cycle currents, flux, supercurrent and the energies, computed by this
package's result class from the stored theta / current / voltage, against the reference's own
values for the same stored quantities (golden fixtures written by tests/golden/make_golden.py).
CPU only: the GPU path's stored quantities are pinned by the parity tests."""
import numpy as np
import pytest

import golden_cases as gc
from pyjjasim_gb300.problem import TimeEvolutionResult

OBSERVABLES = ("phase", "josephson_energy", "supercurrent", "cycle_current", "flux", "magnetic_energy", "potential",
               "capacitive_energy", "energy")


@pytest.mark.parametrize("name", gc.case_names())
def test_observables_match_reference(name):
    z = gc.load(name)
    prob = gc.problem(z)
    res = TimeEvolutionResult(prob, z["theta"], z["current"], z["voltage"])
    for obs in OBSERVABLES:
        got, ref = getattr(res, "get_" + obs)(), z["obs_" + obs]
        assert got.shape == ref.shape, obs
        scale = max(1.0, float(np.abs(ref).max()))
        err = float(np.abs(got - ref).max()) if ref.size else 0.0
        assert err <= 1e-11 * scale, f"{obs}: max abs err {err:.3e}"


def test_observables_select_time_points_and_zero_components():
    z = gc.load("c1_square10_dc")   # no capacitance, no inductance
    prob = gc.problem(z)
    res = TimeEvolutionResult(prob, z["theta"], z["current"], z["voltage"])
    steps = np.flatnonzero(prob.store_time_steps)[[0, 3, 7]]
    assert np.array_equal(res.get_phase(steps), z["obs_phase"][:, :, [0, 3, 7]])
    assert not res.get_capacitive_energy().any() and not res.get_magnetic_energy().any()
    assert res.get_potential(steps).shape == (prob.get_circuit()._Nn(), 1, 3)
