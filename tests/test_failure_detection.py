"""Failure detection without faulting the GPU: a run that diverges is reported, not returned.

The reference raises on bad shapes and types (time_evolution.py:614-628) but lets a diverging
run return NaN phases. The GPU core's update kernel sets a device flag when a new phase is
NaN or +-inf; the plan check that every synchronisation of the Python layer runs turns it into
JJAError code 4 (JJA_ERR_NONFINITE) and clears it, so the plan stays usable. The failures
here are made on the host (NaN or inf in an input); nothing traps or faults on the device.
"""
import numpy as np
import pytest

from pyjjasim_gb300 import SquareArray, TimeEvolutionProblem
from pyjjasim_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _problem(c, Is, **kw):
    return TimeEvolutionProblem(c, time_step=0.05, time_step_count=80, current_sources=Is, external_flux=0.1,
                                store_time_steps=[79], **kw)


def test_nan_input_is_reported_and_the_plan_stays_usable():
    c = SquareArray(9, 7)
    W = 5
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.2, 1.2, W)[None, :, None]
    bad = np.array(Is, dtype=np.float64, copy=True)
    bad[3, 2, 0] = np.nan                       # one junction of one problem
    with pytest.raises(N.JJAError) as e:
        _problem(c, bad).compute()
    assert e.value.code == 4 and "non-finite" in str(e.value)
    # the same circuit and plan afterwards: the flag was cleared, a good run passes
    res = _problem(c, Is).compute()
    assert np.all(np.isfinite(res.get_theta()))


def test_infinite_initial_phase_is_reported():
    c = SquareArray(6, 6)
    th = np.zeros((c.junction_count(), 2))
    th[0, 1] = np.inf
    Is = c.current_base(0.0)[:, None, None] * np.array([0.3, 0.6])[None, :, None]
    with pytest.raises(N.JJAError) as e:
        _problem(c, Is, config_at_minus_1=th, config_at_minus_2=th).compute(use_graph=True)
    assert e.value.code == 4
