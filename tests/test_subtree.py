"""Subtree sweeps: the bottom of the elimination tree solved one warp per (subtree, 32 problems)
in shared memory (k_subtree), before the forward levels and after the backward ones.

CPU: the schedule with subtrees builds and passes its dataflow check on several lattices and
orderings; subtrees take the place of most bottom-level items; the size bound is validated.
GPU: face solves against scipy's sparse direct solve (relative 1e-11) with subtrees of several
sizes, partial warps (W not a multiple of 32) and concurrent problem groups; trajectories with
and without subtrees agree to 1e-11 relative (only the summation order differs).
"""
import numpy as np
import pytest
import scipy.sparse.linalg

from pyjjasim_gb300 import TimeEvolutionProblem, backend
from pyjjasim_gb300 import _native as N
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray

LATTICES = {"square": SquareArray, "honeycomb": HoneycombArray, "triangular": TriangularArray}


def _factor(c, W, ordering):
    return P.get_factor(c, 0.05, nd_leaf=8, ordering=ordering)[0]


@pytest.mark.parametrize("lattice,n,ordering", [("square", 64, "nd"), ("square", 96, "mmd"),
                                                ("honeycomb", 40, "nd"), ("triangular", 48, "mmd")])
def test_schedule_with_subtrees(lattice, n, ordering):
    f = _factor(LATTICES[lattice](n, n), 64, ordering)
    n_off = f.check_schedule(64, {"subtree_rows": -1})
    for rows in (8, 32, 64):
        n_on = f.check_schedule(64, {"subtree_rows": rows})
        assert n_on[0] < n_off[0] and n_on[1] <= n_off[1]
    # below 32 problems per warp the subtrees go into packs of one shape (fewer level items)
    assert f.check_schedule(8, {"subtree_rows": 32})[0] < f.check_schedule(8, {"subtree_rows": -1})[0]


def test_default_takes_subtrees_where_the_launch_is_wide():
    # SquareArray(128,128): about 1000 subtrees, so W = 512 (16 warps each) takes them by default
    # and W = 32 (one warp each, fewer than 152 x 16 warps in all) does not
    f = _factor(SquareArray(128, 128), 512, "mmd")
    assert f.check_schedule(512, {}) == f.check_schedule(512, {"subtree_rows": 32})
    assert f.check_schedule(512, {}) != f.check_schedule(512, {"subtree_rows": -1})
    assert f.check_schedule(32, {}) == f.check_schedule(32, {"subtree_rows": -1})


def test_subtree_rows_bound():
    f = _factor(SquareArray(16, 16), 32, "nd")
    with pytest.raises(N.JJAError):
        f.check_schedule(32, {"subtree_rows": 65})


def _rhs(K, W, seed):
    return np.random.default_rng(seed).standard_normal((K.shape[0], W))


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,n,W,ordering", [("square", 128, 512, "mmd"), ("square", 64, 48, "nd"),
                                                  ("honeycomb", 40, 32, "nd"), ("triangular", 48, 96, "mmd")])
@pytest.mark.parametrize("rows", [0, 8, 64])
def test_subtree_solve_matches_scipy(lattice, n, W, ordering, rows):
    c = LATTICES[lattice](n, n)
    c.set_inductance(0.03)
    A, K = P.face_matrix(c, 0.05)
    b = _rhs(K, W, n + W + rows)
    x = backend.solve_faces(c, 0.05, b, ordering=ordering, tuning={"subtree_rows": rows})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())


@pytest.mark.parametrize("W", [2, 3, 8, 16])
def test_small_w_schedule_packs_subtrees_by_shape(W):
    # below 32 problems per warp: subtrees of one shape share a warp, 32 / WB of them
    f = _factor(SquareArray(96, 96), W, "nd")
    n_off = f.check_schedule(W, {"subtree_rows": -1})
    n_on = f.check_schedule(W, {"subtree_rows": 16})
    assert n_on[0] < n_off[0] and n_on[1] < n_off[1]


@pytest.mark.gpu
@pytest.mark.parametrize("W", [2, 3, 8, 16])
@pytest.mark.parametrize("lattice,n,ordering", [("square", 96, "nd"), ("honeycomb", 40, "mmd")])
def test_small_w_subtree_packs_solve_matches_scipy(lattice, n, ordering, W):
    c = LATTICES[lattice](n, n)
    c.set_inductance(0.03)
    A, K = P.face_matrix(c, 0.05)
    b = _rhs(K, W, n + W)
    x = backend.solve_faces(c, 0.05, b, ordering=ordering, tuning={"subtree_rows": 16})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())


def test_w1_schedule_packs_subtrees_by_shape():
    # W = 1: subtrees of one shape share a warp (32 per warp); the remaining levels shrink
    f = _factor(SquareArray(96, 96), 1, "nd")
    n_off = f.check_schedule(1, {"subtree_rows": -1})
    for rows in (16, 32, 64):
        n_on = f.check_schedule(1, {"subtree_rows": rows})
        assert n_on[0] < n_off[0] and n_on[1] < n_off[1]
    # by default only where the packs fill 152 x 4 warps: not for this single array
    assert f.check_schedule(1, {}) == n_off


@pytest.mark.gpu
@pytest.mark.parametrize("lattice,n,ordering", [("square", 96, "nd"), ("honeycomb", 40, "mmd"),
                                                ("triangular", 48, "nd")])
@pytest.mark.parametrize("rows", [0, 16, 64, -1])
def test_w1_subtree_packs_solve_matches_scipy(lattice, n, ordering, rows):
    c = LATTICES[lattice](n, n)
    c.set_inductance(0.03)
    A, K = P.face_matrix(c, 0.05)
    b = _rhs(K, 1, n + rows)[:, 0]
    x = backend.solve_faces(c, 0.05, b, ordering=ordering, tuning={"subtree_rows": rows})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())


@pytest.mark.gpu
def test_w1_ragged_union_with_and_without_subtree_packs():
    from pyjjasim_gb300.ragged import RaggedBatch
    probs = []
    for k, lat in enumerate((SquareArray, HoneycombArray, TriangularArray, SquareArray)):
        cc = lat(24 + 6 * k, 20 + 4 * k)
        Is = cc.current_base(0.0)[:, None, None] * np.array([0.7 + 0.2 * k])[None, :, None]
        probs.append(TimeEvolutionProblem(cc, time_step=0.05, time_step_count=120, current_sources=Is,
                                          external_flux=0.15, store_time_steps=[119]))
    rb = RaggedBatch(probs, parts=1)
    th_on = [r.get_theta() for r in rb.compute(tuning={"subtree_rows": 32})]
    th_off = [r.get_theta() for r in rb.compute(tuning={"subtree_rows": -1})]
    for a, b in zip(th_on, th_off):
        assert float(np.abs(a - b).max()) <= 1e-11 * max(1.0, float(np.abs(b).max()))


@pytest.mark.gpu
def test_trajectories_with_and_without_subtrees_agree():
    c = SquareArray(48, 48)
    c.set_capacitance(0.3)
    W, Nt = 288, 150           # two problem groups; the last warp of each group partly idle
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.2, 1.8, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, current_sources=Is, external_flux=0.2,
                                store_time_steps=[Nt // 2, Nt - 1])
    mask = prob.store_time_steps
    th_on, _ = backend.time_evolution_core(prob, mask, mask, tuning={"subtree_rows": 32})
    th_off, _ = backend.time_evolution_core(prob, mask, mask, tuning={"subtree_rows": -1})
    scale = max(1.0, float(np.abs(th_off).max()))
    assert float(np.abs(th_on - th_off).max()) <= 1e-11 * scale


def _python_subtrees(f, max_rows):
    """The subtree selection restated from the factor's supernode table: a supernode qualifies
    when its subtree's columns plus its own off-diagonal rows are at most max_rows, no member is
    wider than 8 columns, and the staged F values and row maps stay within 2048 and 4096 entries;
    the subtrees are the qualifying supernodes whose parent does not qualify. The others are
    re-levelled: level 0 when no child remains outside a subtree, else 1 + the largest child level."""
    sn = f.supernodes()
    k, m, par = sn["k"].astype(np.int64), sn["m"].astype(np.int64), sn["parent"]
    ns = len(k)
    cols, fl, ll, kmax, cnt = k.copy(), (k + m) * k, m.copy(), k.copy(), np.ones(ns, np.int64)
    for s in range(ns):
        p = par[s]
        if p >= 0:
            cols[p] += cols[s]; fl[p] += fl[s]; ll[p] += ll[s]; kmax[p] = max(kmax[p], kmax[s]); cnt[p] += cnt[s]
    ok = (cols + m <= max_rows) & (kmax <= 8) & (fl <= 2048) & (ll <= 4096)
    roots = [s for s in range(ns) if ok[s] and (par[s] < 0 or not ok[par[s]])]
    level = np.zeros(ns, np.int64)
    top = -1
    for s in range(ns):
        if ok[s]:
            continue
        top = max(top, level[s])
        if par[s] >= 0:
            level[par[s]] = max(level[par[s]], level[s] + 1)
    return len(roots), int(ok.sum()), int(max((cols + m)[roots], default=0)), top + 1


@pytest.mark.parametrize("lattice,n,ordering,W,rows", [("square", 128, "mmd", 512, 32), ("square", 64, "nd", 64, 24),
                                                       ("honeycomb", 40, "nd", 32, 48), ("triangular", 48, "mmd", 8, 32),
                                                       ("square", 96, "nd", 1, 16)])
def test_schedule_stats_match_the_subtree_rule(lattice, n, ordering, W, rows):
    f = _factor(LATTICES[lattice](n, n), W, ordering)
    st = f.schedule_stats(W, {"subtree_rows": rows})
    n_sub, members, max_rows, levels = _python_subtrees(f, rows)
    assert (st["n_subtrees"], st["n_subtree_members"], st["max_subtree_rows"], st["n_levels"]) == \
        (n_sub, members, max_rows, levels)
    if W < 32:      # packs of 32 / WB subtrees of one shape, one item per pack and problem block
        wb = 1 << max(0, (W - 1).bit_length())
        assert st["n_pack_shapes"] <= n_sub
        assert st["n_pack_items"] >= -(-n_sub // (32 // wb)) * (-(-W // wb))
    else:
        assert st["n_pack_items"] == 0
    off = f.schedule_stats(W, {"subtree_rows": -1})
    assert off["n_subtrees"] == 0 and off["n_levels"] == f.stats["n_levels"]
    assert (st["n_fwd_items"], st["n_bwd_items"]) == f.check_schedule(W, {"subtree_rows": rows})
