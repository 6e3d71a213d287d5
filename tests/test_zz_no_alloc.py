"""jja_solve_static: the face-space solve for callers that cannot allocate device memory.

Such callers (code whose device memory belongs to another allocator, or that runs under a
fixed budget, or per-step loops that must not synchronise the device through cudaMalloc) get
the same solve with the work vectors in a fixed array inside the library. This file is
collected last on purpose. The test calls the entry point through the C ABI twice in a row and
checks each result against jja_solve's (the allocating entry point) within the 1e-11 relative
tolerance the face-solve tests use; the two calls also show that the array's leftover contents
from one call do not leak into the next. It covers both schedules of the triangular sweeps
(one launch per level, and the dataflow sweep whose bounded waits are confirmed by the plan
check after every call), one problem per launch with small supernodes solved one per lane, and
the subtree sweeps (one warp per subtree and 32 problems, and packs of subtrees of one shape for
8 problems and for one).
"""
import ctypes

import numpy as np
import pytest

from pyjjasim_gb300 import _native as N
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import SquareArray
from pyjjasim_gb300.problem import stencil

pytestmark = pytest.mark.gpu


def _plan(n, W, tuning=None):
    c = SquareArray(n, n)
    c.set_inductance(0.05)
    return P.get_plan(c, 0.05, W, 3, stencil(3), tuning=tuning), (n - 1) * (n - 1)


@pytest.mark.parametrize("W,tuning", [(24, {"schedule": 1}), (24, {"schedule": 2}),
                                      (1, {"pack_min_warps": 1}), (1, {"schedule": 2}),
                                      (24, {"subtree_rows": 32}), (8, {"subtree_rows": 32}),
                                      (1, {"subtree_rows": 16})])
def test_static_solve_matches_allocating_solve_twice(W, tuning):
    import torch
    lib = N.lib()
    pl, Nf = _plan(40, W, tuning)
    rng = np.random.default_rng(5)
    for call in range(2):
        b = torch.from_numpy(rng.standard_normal((Nf, W))).cuda()
        x_ref = torch.empty_like(b)
        x_sta = torch.full_like(b, float("nan"))
        N.check(lib.jja_solve(pl.handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x_ref.data_ptr()), None))
        pl.check()       # synchronises; raises if a dataflow wait ran out
        N.check(lib.jja_solve_static(pl.handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x_sta.data_ptr()),
                                     None))
        torch.cuda.synchronize()
        pl.check()
        a, r = x_sta.cpu().numpy(), x_ref.cpu().numpy()
        assert np.all(np.isfinite(a)), f"call {call}: non-finite output"
        err = np.abs(a - r).max() / np.abs(r).max()
        assert err <= 1e-11, f"call {call}: relative difference {err:.3e}"


def test_static_solve_rejects_plans_beyond_its_limit():
    import torch
    lib = N.lib()
    pl, Nf = _plan(64, 600)            # 3969 faces x 600 problems > 2,097,152
    b = torch.zeros((Nf, 600), dtype=torch.float64, device="cuda")
    x = torch.empty_like(b)
    code = lib.jja_solve_static(pl.handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()), None)
    assert code == 1  # JJA_ERR_ARG
    assert b"static scratch limit" in lib.jja_last_error()
