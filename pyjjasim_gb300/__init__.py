"""pyjjasim_gb300 — GB300-native (sm_103a, FP64) time-evolution core for pyjjasim.

Drop-in replacement of the reference's RCSJ time-stepping hot path
(pyjjasim time_evolution.py:461-582). Two ways to use it:

* this package's own API, which mirrors the reference's::

      from pyjjasim_gb300 import SquareArray, TimeEvolutionProblem
      a = SquareArray(128, 128)
      prob = TimeEvolutionProblem(a, time_step=0.05, time_step_count=10000,
                                  current_sources=a.current_base(0)[:, None, None] * bias[None, :, None],
                                  external_flux=0.25)
      result = prob.compute()            # runs on the GPU

* the reference package itself, with its core swapped in (``install``)::

      import pyjjasim, pyjjasim_gb300
      pyjjasim_gb300.install(pyjjasim)   # TimeEvolutionProblem.compute() now steps on the GPU
"""
from .circuit import Circuit, HoneycombArray, SquareArray, TriangularArray
from .problem import (CurrentNotStored, DataAtTimepointNotStored, DefaultCPR, ThetaNotStored, TimeEvolutionProblem,
                      TimeEvolutionResult, VoltageNotStored, time_evolution)
from .static import NewtonIterInfo, StaticConfiguration, StaticProblem

__all__ = ["Circuit", "SquareArray", "HoneycombArray", "TriangularArray", "DefaultCPR", "TimeEvolutionProblem",
           "TimeEvolutionResult", "time_evolution", "install", "uninstall", "time_evolution_core",
           "ThetaNotStored", "CurrentNotStored", "VoltageNotStored", "DataAtTimepointNotStored",
           "StaticProblem", "StaticConfiguration", "NewtonIterInfo"]


def time_evolution_core(problem, th_store_mask, I_store_mask, **options):
    """GPU core with the reference's signature (time_evolution.py:461)."""
    from .backend import time_evolution_core as core
    return core(problem, th_store_mask, I_store_mask, **options)


_saved = {}


def install(pyjjasim_module, **options):
    """Route the reference's ``time_evolution_core`` to the GPU core.

    ``pyjjasim_module`` is the imported reference package (or its ``time_evolution``
    submodule). ``options`` (e.g. ``noise="numpy"``) are passed to every call.
    The reference's ``time_evolution()`` (voltage post-processing, masks) and
    ``TimeEvolutionResult`` stay the reference's own.
    """
    te = getattr(pyjjasim_module, "time_evolution", pyjjasim_module)
    if not hasattr(te, "time_evolution_core"):
        import importlib
        te = importlib.import_module(pyjjasim_module.__name__ + ".time_evolution")
    if te not in _saved:
        _saved[te] = te.time_evolution_core

    def core(problem, th_store_mask, I_store_mask):
        return time_evolution_core(problem, th_store_mask, I_store_mask, **options)

    te.time_evolution_core = core
    return te


def uninstall():
    """Restore every module patched by ``install``."""
    for te, fn in list(_saved.items()):
        te.time_evolution_core = fn
        del _saved[te]
