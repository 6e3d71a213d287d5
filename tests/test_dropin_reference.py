"""The drop-in switch against the reference package itself (CPU; skipped where its sources are
absent, e.g. on machines that only run the GPU tests).

``pyjjasim_gb300.install(pyjjasim)`` replaces the reference's ``time_evolution_core``
(time_evolution.py:461), which its ``time_evolution()`` (:443) calls from
``TimeEvolutionProblem.compute()`` (:303-307). These tests import the reference (with the
shim of tests/golden/make_golden.py) and check, on the reference's OWN problem and circuit
objects:
* the GPU core's host staging (everything before its first CUDA call) reads them: sizes,
  initial phases, sources with the reference's zero and time-dependence tests;
* the host factorisation of the reference circuit's face-space matrix solves like scipy, and
  the GPU work-item schedule for it builds and passes its dataflow check;
* after ``install``, the reference's ``compute()`` dispatches to this package's core with the
  reference's problem object, and its results (through a core that stages the problem and then
  steps it with the oracle, as no GPU is here) equal the uninstalled reference's; ``uninstall``
  restores the reference;
* without a GPU the installed core fails loudly (no CPU fallback).
"""
import importlib.util
import os

import numpy as np
import pytest
import scipy.sparse.linalg

import pyjjasim_gb300 as G
from oracle import rcsj_oracle
from pyjjasim_gb300 import backend
from pyjjasim_gb300 import plan as P

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("PYJJASIM_REFERENCE", "/root/reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")


@pytest.fixture(scope="module")
def pj():
    import sys
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ref = mg.import_reference(REF)
    for m in mg.MATPLOTLIB_STUBS:       # the reference holds its own references to the stubs
        sys.modules.pop(m, None)
    return ref


def _ref_problem(pj, Nt=120):
    a = pj.SquareArray(7, 6)
    a.set_capacitance(0.3)
    a.set_inductance(0.2)
    W = 3
    Is = a.current_base(0.0)[:, None, None] * np.linspace(0.4, 1.4, W)[None, :, None]
    f = np.random.default_rng(2).uniform(0.0, 0.3, (a.face_count(), W, 1))
    return pj.TimeEvolutionProblem(a, time_step=0.05, time_step_count=Nt, current_sources=Is, external_flux=f,
                                   store_time_steps=np.arange(0, Nt, 10))


def test_host_staging_reads_the_reference_problem(pj):
    p = _ref_problem(pj)
    a = p.get_circuit()
    assert type(p).__module__ == "pyjjasim.time_evolution"
    st = backend.HostStage(p)
    assert (st.Nj, st.Nf, st.W, st.width, st.Nt) == (a._Nj(), a._Nf(), 3, 3, 120)
    assert all(z for z in st.hist0_zero) and all(h.shape == (a._Nj(), 3) for h in st.hist0)
    src = st.sources
    assert not src["Is"]["zero"] and not src["f"]["zero"] and src["Vs"]["zero"] and src["T"]["zero"]
    assert not any(s["timedep"] for s in src.values())
    np.testing.assert_array_equal(src["Is"]["getter"](0), p._Is(0))
    # a time-dependent temperature is never zero-tested (time_evolution.py:512-519)
    p2 = pj.TimeEvolutionProblem(a, time_step=0.05, time_step_count=10, temperature=np.zeros((a._Nj(), 1, 10)))
    assert backend.HostStage(p2).sources["T"]["timedep"] and not backend.HostStage(p2).sources["T"]["zero"]


def test_host_factor_of_the_reference_circuit(pj):
    a = _ref_problem(pj).get_circuit()
    f, A, _ = P.get_factor(a, 0.05, ordering="nd")
    _, K = P.face_matrix(a, 0.05)
    b = np.random.default_rng(3).standard_normal((K.shape[0], 4))
    x = f.solve_host(b)
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    assert np.abs(x - ref).max() <= 1e-11 * np.abs(ref).max()
    n_fwd, n_bwd = f.check_schedule(3)
    assert n_fwd > 0 and n_bwd > 0


def test_install_routes_the_reference_compute(pj, monkeypatch):
    expected = _ref_problem(pj).compute()            # the reference, uninstalled
    seen = []

    def staged_oracle_core(problem, th_store_mask, I_store_mask, **options):
        seen.append(type(problem))
        backend.HostStage(problem)                    # the GPU core's host side accepts it
        return rcsj_oracle.evolve(problem, th_store_mask, I_store_mask)

    monkeypatch.setattr(backend, "time_evolution_core", staged_oracle_core)
    te = G.install(pj)
    try:
        assert te.time_evolution_core is not G._saved[te]
        got = _ref_problem(pj).compute()
    finally:
        G.uninstall()
    assert seen == [pj.TimeEvolutionProblem]
    assert te.time_evolution_core.__module__ == "pyjjasim.time_evolution"
    for name in ("get_theta", "get_current", "get_voltage"):
        np.testing.assert_allclose(getattr(got, name)(), getattr(expected, name)(), rtol=0, atol=1e-12)
    np.testing.assert_array_equal(got.get_vortex_configuration(), expected.get_vortex_configuration())


def test_installed_core_fails_loudly_without_a_gpu(pj):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    G.install(pj)
    try:
        with pytest.raises(RuntimeError, match="CUDA GPU"):
            _ref_problem(pj).compute()
    finally:
        G.uninstall()
