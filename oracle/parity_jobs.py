"""Oracle runs of the benchmark's workloads at their real sizes (TEST INFRASTRUCTURE ONLY).

The checker side of the full-size parity checks: only tests/ and bench.py call these, and only
to compare the GPU results with; nothing here is timed as the product or shipped with it. Each
function builds its problem with the package's own lattice and problem classes (the inputs the
GPU run gets) and runs ``rcsj_oracle.evolve`` (the restatement of pyjjasim's
time_evolution_core, time_evolution.py:461-582) on it. The functions are picklable top-level
calls so a caller can run them in worker processes started with ``spawn`` (``pool``), in
parallel with its GPU work.
"""
import contextlib
import os

import numpy as np

# the batched IV sweep (SquareArray(128, 128), f = 0.25, dt = 0.05, T = 0, DC bias on current_base(0))
IV_N, IV_F, IV_DT = 128, 0.25, 0.05
# the large single array (SquareArray(1024, 1024), beta_C = 0.5, L = 0.05, f = 0.1, dt = 0.05)
LARGE_N, LARGE_C, LARGE_L, LARGE_F, LARGE_DT = 1024, 0.5, 0.05, 0.1, 0.05


def mmd_factorize(K):
    """SuperLU with the MMD(A^T + A) column order instead of the reference's default (COLAMD):
    the same LU algorithm with a different summation order."""
    import scipy.sparse
    import scipy.sparse.linalg
    return scipy.sparse.linalg.splu(scipy.sparse.csc_matrix(K), permc_spec="MMD_AT_PLUS_A").solve


def _theta_at(problem, store, factorize=None):
    from . import rcsj_oracle
    Nt = problem._Nt()
    mask = np.zeros(Nt, bool)
    mask[list(store)] = True
    th, _ = rcsj_oracle.evolve(problem, mask, np.zeros(Nt, bool), factorize=factorize)
    return th[:, :, problem.stencil_width - 1:]          # (Nj, W, len(store)), steps ascending


def iv_sweep_problem(G, bias, Nt, store=None):
    """W = len(bias) problems of the batched IV sweep, bias current_base(0) * bias[w], phases
    stored at the steps ``store`` (default: the last)."""
    a = G.SquareArray(IV_N, IV_N)
    Is = a.current_base(0.0)[:, None, None] * np.asarray(bias, np.float64)[None, :, None]
    return G.TimeEvolutionProblem(a, time_step=IV_DT, time_step_count=Nt, current_sources=Is, external_flux=IV_F,
                                  store_time_steps=[Nt - 1] if store is None else list(store), store_voltage=False,
                                  store_current=False)


def iv_sweep_theta(bias, Nt, store, alt_order=False):
    """Oracle phases (Nj, len(store)) of ONE problem of the IV sweep at the steps ``store``;
    ``alt_order``: factorise with the MMD order (rounding-sensitivity run)."""
    import pyjjasim_gb300 as G
    p = iv_sweep_problem(G, [bias], Nt)
    return _theta_at(p, store, mmd_factorize if alt_order else None)[:, 0, :]


def large_array_problem(G, bias, Nt, base=None, temperature=0.0):
    """SquareArray(1024, 1024), C = 0.5, L = 0.05, f = 0.1, bias current_base(0) * bias[w] (the
    reference's current_base, passed in as ``base`` when already computed)."""
    a = G.SquareArray(LARGE_N, LARGE_N)
    a.set_capacitance(LARGE_C)
    a.set_inductance(LARGE_L)
    if base is None:
        base = a.current_base(0.0)
    Is = base[:, None, None] * np.asarray(bias, np.float64)[None, :, None]
    return G.TimeEvolutionProblem(a, time_step=LARGE_DT, time_step_count=Nt, current_sources=Is,
                                  external_flux=LARGE_F, temperature=temperature, store_time_steps=[Nt - 1],
                                  store_voltage=False, store_current=False)


def large_array_theta(bias, Nt, store):
    """Oracle phases (Nj, W, len(store)) of the large single array at T = 0, and the
    current_base(0) vector the problem was built with (so the GPU side reuses it)."""
    import pyjjasim_gb300 as G
    a = G.SquareArray(LARGE_N, LARGE_N)
    base = a.current_base(0.0)
    p = large_array_problem(G, bias, Nt, base=base)
    return _theta_at(p, store), base


@contextlib.contextmanager
def _single_threaded_blas():
    keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = "1"
    try:
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def pool(n):
    """A pool of ``n`` worker processes started with ``spawn`` (safe next to a CUDA context in
    the caller) whose BLAS runs single-threaded (one job per core)."""
    import multiprocessing
    with _single_threaded_blas():
        return multiprocessing.get_context("spawn").Pool(max(1, n))
