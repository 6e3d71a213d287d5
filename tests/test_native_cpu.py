"""C ABI library: loads, exports every declared symbol, and its host factorisation is right.

These run without a GPU: the host factorisation and the host diagnostic solve need none.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg

from pyjjasim_gb300 import _native as N
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "jja_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jja_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    decl = declared_symbols()
    assert decl, "no declarations parsed"
    missing = [s for s in decl if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    # and the ctypes binding covers exactly the declared surface
    assert sorted(N.SIGNATURES) == decl


@pytest.mark.parametrize("make", [lambda: SquareArray(12, 9), lambda: HoneycombArray(5, 4),
                                  lambda: TriangularArray(6, 7), lambda: SquareArray(40, 40)])
@pytest.mark.parametrize("L", [0.0, 0.3])
def test_host_factor_solves_face_matrix(make, L):
    c = make()
    c.set_capacitance(0.5)
    c.set_inductance(L)
    A, K = P.face_matrix(c, 0.05)
    f = P.HostFactor(K, coords=P._coords(c))
    b = np.random.default_rng(1).standard_normal((K.shape[0], 3))
    x = f.solve_host(b)
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
    st = f.stats
    assert st["n"] == K.shape[0] and st["n_levels"] >= 1 and st["nnz_L"] >= K.shape[0]
    perm = f.perm()
    assert sorted(perm.tolist()) == list(range(K.shape[0]))


def test_host_factor_without_coordinates_and_with_user_perm():
    c = SquareArray(15, 11)
    A, K = P.face_matrix(c, 0.1)
    b = np.random.default_rng(2).standard_normal(K.shape[0])
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    for kw in (dict(coords=None), dict(perm=np.arange(K.shape[0])[::-1].copy())):
        x = P.HostFactor(K, **kw).solve_host(b)
        assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()


def test_factor_rejects_indefinite_and_bad_perm():
    K = scipy.sparse.csc_matrix(np.array([[1.0, 2.0], [2.0, 1.0]]))
    with pytest.raises(N.JJAError) as e:
        P.HostFactor(K)
    assert e.value.code == 2  # JJA_ERR_NOT_SPD
    K = scipy.sparse.csc_matrix(np.eye(3) * 2.0)
    with pytest.raises(N.JJAError):
        P.HostFactor(K, perm=np.array([0, 0, 1]))


def test_nested_dissection_fill_is_bounded():
    # ND on a square lattice keeps nnz(L) near the n^2 log n regime (128x128 nodes: ~4.6e5)
    c = SquareArray(128, 128)
    A, K = P.face_matrix(c, 0.05)
    st = P.HostFactor(K, coords=P._coords(c)).stats
    assert st["nnz_L"] < 6.0e5
    assert st["n_levels"] <= 30


def test_fixed_point_sine_on_host():
    """The junction kernels' sine and cosine (64-bit fixed point + FP32, no FP64 instruction),
    run on the host from the same source: within 1.2e-16 absolute of numpy for |x| < 2^62; near
    zeros of sine within 1e-18 absolute (a few units of the fixed point's 2^-62) plus 2 ulps;
    x itself below 2^-27; NaN from 2^62 on and for inf and NaN."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 400000), rng.uniform(-4, 4, 200000),
                        np.arange(-3000, 3000) * (np.pi / 2048) + rng.uniform(-1e-9, 1e-9, 6000),
                        np.arange(-3000, 3000) * (np.pi / 2) + rng.uniform(-1e-7, 1e-7, 6000),
                        10.0 ** rng.uniform(-12, 18.6, 300000), rng.uniform(-2e5, 2e5, 100000),
                        np.array([0.0, -0.0, 1e-300, 2.0 ** -27, -(2.0 ** -27), np.pi, 1e5, 199999.99, 2e5, 3e5,
                                  -7e6, 2.0 ** 62 * (1 - 2.0 ** -53), 2.0 ** 62, -1e300, np.inf, -np.inf, np.nan])])
    s, c = np.empty_like(x), np.empty_like(x)
    N.check(N.lib().jja_sin_host(N.ptr(x), N.ptr(s), N.ptr(c), x.size))
    with np.errstate(invalid="ignore"):
        rs, rc = np.sin(x), np.cos(x)
    fin = np.abs(x) < 2.0 ** 62     # beyond, and for inf and NaN: NaN
    assert np.all(np.isnan(s[~fin])) and np.all(np.isnan(c[~fin]))
    assert np.abs(s - rs)[fin].max() <= 1.2e-16 and np.abs(c - rc)[fin].max() <= 1.2e-16
    tiny = np.abs(x) < 2.0 ** -27
    assert np.array_equal(s[tiny], x[tiny]) and np.all(c[tiny] == 1.0)
    xf = np.where(fin, x, 0.0)
    near = fin & (np.abs(xf - np.round(xf / np.pi) * np.pi) < np.pi / 4096) & (np.abs(xf) < 2e5)
    assert near.sum() > 1000 and np.all(np.abs(s - rs)[near] <= 1e-18 + 2.3e-16 * np.abs(rs[near]))


def test_auto_ordering_policy():
    # minimum degree only where the step is FP64-bound (lots of face-problems) and SuperLU's
    # host ordering run stays cheap; explicit orderings pass through
    assert P.resolve_ordering("auto", 512, 127 * 127) == "mmd"
    assert P.resolve_ordering("auto", 64, 63 * 63) == "nd"
    assert P.resolve_ordering("auto", 1, 255 * 255) == "nd"
    assert P.resolve_ordering("auto", 8, 1023 * 1023) == "nd"
    assert P.resolve_ordering("nd", 512, 127 * 127) == "nd" and P.resolve_ordering("mmd", 1, 10) == "mmd"


def test_plan_create_without_gpu_reports_cuda_error():
    # creating a device plan must fail loudly (no CPU fallback) when no GPU is present
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    c = SquareArray(5, 5)
    A, K = P.face_matrix(c, 0.05)
    f = P.HostFactor(K)
    with pytest.raises(N.JJAError) as e:
        P.DevicePlan(c, f, A, 2, 0.05, 3, ((1.0, -1.0, 0.0), (1.0, -2.0, 1.0)))
    assert e.value.code == 3  # JJA_ERR_CUDA


@pytest.mark.parametrize("make", [lambda: SquareArray(128, 128), lambda: HoneycombArray(20, 17),
                                  lambda: TriangularArray(30, 21), lambda: SquareArray(7, 5)])
@pytest.mark.parametrize("ordering", ["nd", "mmd"])
@pytest.mark.parametrize("W,tuning", [(1, None), (1, {"pack_rows": -1}), (1, {"pack_min_warps": 1}),
                                      (1, {"pack_rows": 64, "pack_min_warps": 1}),
                                      (8, {"rows_per_lane": 8}), (64, {"rhs_block": 16}),
                                      (512, None), (512, {"rows_per_lane": 2, "min_piece": 4,
                                                          "target_warps": 152 * 200}), (3, {"schedule": 2})])
def test_dataflow_schedule_waits_only_on_earlier_items(make, ordering, W, tuning):
    """The work-item schedule of both sweeps (built on the host exactly as the GPU plan builds it)
    is a valid dataflow order: no item waits for a later item, and every wait count equals the
    number of items that count towards it. A violation could make warps wait for items no
    running warp holds."""
    c = make()
    A, K = P.face_matrix(c, 0.05)
    coords, perm = P.fill_reducing_order(K, ordering, c)
    f = P.HostFactor(K, coords=coords, perm=perm)
    nf, nb = f.check_schedule(W, tuning)          # with the library's subtree sweeps
    assert nf >= 0 and nb >= 0
    # without subtrees every supernode has a level item, or a place in a W = 1 pack of <= 32
    flat = dict(tuning or {}, subtree_rows=-1)
    nf, nb = f.check_schedule(W, flat)
    ns = f.stats["n_supernodes"]
    packed = W == 1 and flat.get("pack_rows", 0) >= 0
    least = -(-ns // 32) if packed else ns
    assert nf >= least and nb >= least
    if packed and flat.get("pack_min_warps") == 1 and ns > 64:   # packs on every level
        nf1, nb1 = f.check_schedule(W, {"pack_rows": -1, "subtree_rows": -1})
        assert nf < nf1 and nb < nb1


def test_ctypes_structs_match_the_header():
    """Field names and order of the ctypes mirrors equal the C structs in include/jja_gb300.h."""
    text = open(os.path.join(os.path.dirname(__file__), "..", "include", "jja_gb300.h")).read()

    def c_fields(name):
        end = text.index("} " + name + ";")
        start = text.rindex("typedef struct {", 0, end)
        body = re.sub(r"/\*.*?\*/", "", text[start:end], flags=re.S)
        out = []
        for decl in body.split(";")[:-1]:
            decl = decl.replace("typedef struct {", "").strip()
            if not decl:
                continue
            names = decl.split(",")
            first = re.findall(r"(\w+)\s*(?:\[\d+\])?$", names[0].strip())[0]
            out.append(first)
            out.extend(re.findall(r"\**\s*(\w+)", n)[0] for n in names[1:])
        return out

    for cname, pystruct in (("jja_solve_tuning", N.SolveTuning), ("jja_view", N.View), ("jja_state", N.State),
                            ("jja_plan_desc", N.PlanDesc), ("jja_adjoint_args", N.AdjointArgs),
                            ("jja_adjoint_segment_args", N.AdjointSegmentArgs), ("jja_factor_opts", N.FactorOpts),
                            ("jja_factor_stats", N.FactorStats), ("jja_schedule_stats", N.ScheduleStats)):
        assert c_fields(cname) == [f for f, _ in pystruct._fields_], cname


def test_default_launch_shape_rules():
    """The library's defaults equal the explicit settings they stand for: two forward rows per
    lane from W = 8 on arrays of 2^17 faces or more (and from W = 256 everywhere), one below; a
    split target of 152 x 64 warps for 2-16 problems, 152 x 24 otherwise."""
    def sched(n, W, tuning):
        f = P.get_factor(SquareArray(n, n), 0.05, nd_leaf=8, ordering="nd")[0]
        st = f.schedule_stats(W, dict(tuning, subtree_rows=-1))
        return st["n_fwd_items"], st["n_bwd_items"]

    big, small = 400, 256                  # 159 201 and 65 025 faces
    assert sched(big, 8, {}) == sched(big, 8, {"rows_per_lane_fwd": 2, "target_warps": 152 * 64})
    assert sched(big, 8, {}) != sched(big, 8, {"rows_per_lane_fwd": 1, "target_warps": 152 * 64})
    assert sched(small, 8, {}) == sched(small, 8, {"rows_per_lane_fwd": 1, "target_warps": 152 * 64})
    assert sched(small, 1, {}) == sched(small, 1, {"rows_per_lane_fwd": 1, "target_warps": 152 * 24})
    assert sched(small, 512, {}) == sched(small, 512, {"rows_per_lane_fwd": 2, "target_warps": 152 * 24})
