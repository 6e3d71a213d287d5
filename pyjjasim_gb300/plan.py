"""Host-side plan: the face-space matrix, its factor and the device plan, cached.

The reference rebuilds and refactorises K = A (L + diag(1/Cnext)) A^T inside every
time_evolution_core call (time_evolution.py:504-506). Here the factor (host, FP64,
nested dissection + supernodal Cholesky in libjja_gb300) and the device plan (factor
blocks + circuit tables uploaded once) are cached by the content that determines them:
the cycle matrix, R, C, L, dt and the stencil width (and W for the device plan), so
repeated compute() calls on the same circuit (e.g. an annealing schedule or a sweep)
pay the factorisation once.
"""
import ctypes
import hashlib
import threading
from collections import OrderedDict

import numpy as np
import scipy.sparse

from . import _native as N

_FACTORS = OrderedDict()
_PLANS = OrderedDict()
MAX_FACTORS = 4
MAX_PLANS = 4
_CACHE_LOCK = threading.Lock()   # the caches are shared by host threads (ragged parts build in parallel);
                                 # the lock covers lookups and insertions, not the factorisations

# Extrapolation weights of the CPR argument on theta(t-1), theta(t-2), ... (time_evolution.py:547-553)
EXTRAP = {3: (2.0, -1.0), 4: (3.0, -3.0, 1.0), 5: (4.0, -6.0, 4.0, -1.0)}
# launch-shape fields of the triangular solves (jja_solve_tuning)
TUNING_FIELDS = ("rhs_block", "rows_per_lane", "target_warps", "min_piece", "schedule", "rows_per_lane_fwd",
                 "pack_rows", "pack_min_warps", "pdl", "groups", "coop_blocks", "dst_lines",
                 "pack_lanes", "subtree_rows")
SCHEDULES = {"levels": 1, "dataflow": 2, "cooperative": 3}


def _digest(*arrays):
    h = hashlib.blake2b(digest_size=16)
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode() + str(a.shape).encode())
        h.update(a.view(np.uint8).ravel() if a.size else b"")
    return h.hexdigest()


def coefficients(circuit, dt, stencil):
    """Per-junction stencil coefficients (time_evolution.py:472-478, 489, 495, 501)."""
    s1, s2 = stencil
    Rv = 1.0 / (dt * np.asarray(circuit._R(), np.float64))
    Cv = np.asarray(circuit._C(), np.float64) / dt ** 2
    coef = [s1[k] * Rv + s2[k] * Cv for k in range(len(s1))]
    return Rv, Cv, coef


def face_matrix(circuit, dt):
    """K = A (L + diag(1/(Cv + Rv))) A^T as CSC with sorted indices (time_evolution.py:504-505)."""
    A = scipy.sparse.csc_matrix(circuit.get_cycle_matrix()).astype(np.float64)
    Rv = 1.0 / (dt * np.asarray(circuit._R(), np.float64))
    Cv = np.asarray(circuit._C(), np.float64) / dt ** 2
    L = circuit._L()
    L = scipy.sparse.csc_matrix(L) if not scipy.sparse.issparse(L) else L
    K = (A @ (L + scipy.sparse.diags(1.0 / (Cv + Rv), 0)) @ A.T).tocsc()
    K.sum_duplicates()
    K.sort_indices()
    return A, K


class HostFactor:
    """Ordered supernodal Cholesky of K (owned C object)."""

    def __init__(self, K, coords=None, perm=None, nd_leaf=8, max_supernode=0, keep_factor=False, relax_zeros=-1,
                 relax_frac=-1.0):
        L = N.lib()
        n = K.shape[0]
        self.n = n
        colptr = np.ascontiguousarray(K.indptr, np.int64)
        rowind = np.ascontiguousarray(K.indices, np.int32)
        val = np.ascontiguousarray(K.data, np.float64)
        cx = cy = None
        if coords is not None:
            cx = np.ascontiguousarray(coords[0], np.float64)
            cy = np.ascontiguousarray(coords[1], np.float64)
        pm = None if perm is None else np.ascontiguousarray(perm, np.int32)
        opts = N.FactorOpts(nd_leaf, max_supernode, int(keep_factor), int(relax_zeros), float(relax_frac))
        h = ctypes.c_void_p()
        N.check(L.jja_factor_create(n, N.ptr(colptr, ctypes.c_int64), N.ptr(rowind, ctypes.c_int32), N.ptr(val),
                                    N.ptr(cx), N.ptr(cy), N.ptr(pm, ctypes.c_int32), ctypes.byref(opts),
                                    ctypes.byref(h)))
        self.handle = h
        st = N.FactorStats()
        N.check(L.jja_factor_get_stats(h, ctypes.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in N.FactorStats._fields_}

    def perm(self):
        out = np.empty(self.n, np.int32)
        N.check(N.lib().jja_factor_get_perm(self.handle, N.ptr(out, ctypes.c_int32)))
        return out

    def supernodes(self):
        """dict of per-supernode arrays: col0, k, m, level, parent."""
        ns = self.stats["n_supernodes"]
        out = {k: np.empty(ns, np.int32) for k in ("col0", "k", "m", "level", "parent")}
        N.check(N.lib().jja_factor_get_supernodes(self.handle, *(N.ptr(out[k], ctypes.c_int32)
                                                                for k in ("col0", "k", "m", "level", "parent"))))
        return out

    def check_schedule(self, W, tuning=None):
        """Build the GPU work-item schedule for W problems on the host and check its dataflow
        order (raises JJAError otherwise); returns the item counts (forward, backward)."""
        t = dict(tuning or {})
        tu = N.SolveTuning(*(int(t.get(f, 0)) for f in TUNING_FIELDS))
        nf, nb = ctypes.c_int64(0), ctypes.c_int64(0)
        N.check(N.lib().jja_factor_check_schedule(self.handle, int(W), ctypes.byref(tu), ctypes.byref(nf),
                                                  ctypes.byref(nb)))
        return nf.value, nb.value

    def schedule_stats(self, W, tuning=None):
        """dict: the shape of the GPU schedule for W problems (levels, bottom subtrees, subtree
        packs, work items), built on the host as the plan builds it."""
        t = dict(tuning or {})
        tu = N.SolveTuning(*(int(t.get(f, 0)) for f in TUNING_FIELDS))
        st = N.ScheduleStats()
        N.check(N.lib().jja_factor_schedule_stats(self.handle, int(W), ctypes.byref(tu), ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in N.ScheduleStats._fields_}

    def solve_host(self, b):
        """Host solve (diagnostic). b: (n,) or (n, nrhs)."""
        b = np.array(b, dtype=np.float64, order="C", copy=True)
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        N.check(N.lib().jja_factor_solve_host(self.handle, N.ptr(b), nrhs))
        return b

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.jja_factor_destroy(h)
            self.handle = None


def fast_poisson_grid(circuit, K):
    """(mx, my, grid_face, kappa) when the face-space matrix is K = kappa (4 I - adjacency) on an
    mx x my grid of faces with mx + 1 and my + 1 powers of two (up to 1024): a square array with
    equal R and C and a uniform self-inductance, whose K is kappa times the 5-point Laplacian with
    Dirichlet boundaries. Checked entry by entry (relative 1e-12); None otherwise."""
    try:
        cx, cy = circuit.get_face_centroids()
    except Exception:
        return None
    Nf = K.shape[0]
    ux, ix = np.unique(np.round(np.asarray(cx, np.float64), 9), return_inverse=True)
    uy, iy = np.unique(np.round(np.asarray(cy, np.float64), 9), return_inverse=True)
    mx, my = len(ux), len(uy)
    if mx * my != Nf or any(m + 1 > 1024 or (m + 1) & m for m in (mx, my)):
        return None
    grid = np.full(mx * my, -1, np.int64)
    grid[iy * mx + ix] = np.arange(Nf)
    if np.any(grid < 0):
        return None
    Kc = scipy.sparse.coo_matrix(K)
    kappa = float(K.diagonal()[0]) / 4.0
    if not kappa > 0.0:
        return None
    tol = 1e-12 * kappa
    if np.abs(K.diagonal() - 4.0 * kappa).max() > tol:
        return None
    off = Kc.row != Kc.col
    r, c, v = Kc.row[off], Kc.col[off], Kc.data[off]
    neighbour = (np.abs(ix[r] - ix[c]) + np.abs(iy[r] - iy[c])) == 1
    if not np.all(neighbour) or np.abs(v + kappa).max(initial=0.0) > tol:
        return None
    if np.count_nonzero(np.abs(v) > tol) != 2 * (mx * (my - 1) + my * (mx - 1)):
        return None
    return mx, my, np.ascontiguousarray(grid, np.int32), kappa


# "auto" uses the sine transforms for at most this many problems and face-problems (W x Nf). Measured
# on GB300 (device ms per step, transforms / sweeps): 256x256 W = 1 0.066 / 0.158, 128x128 W = 1
# 0.031 / 0.082, W = 8 0.092 / 0.142, W = 16 0.168 / 0.163, W = 64 0.60 / 0.30; 512x512 W = 1
# 0.23 / 0.36; 1024x1024 W = 1 0.85 / 0.79, W = 8 6.3 / 2.9; 64x64 W = 64 0.150 / 0.129
FAST_POISSON_MAX_W = 8
FAST_POISSON_MAX_WORK = 1 << 18


class DevicePlan:
    """Circuit tables + factor uploaded for W problems (owned C object)."""

    def __init__(self, circuit, factor, A, W, dt, stencil_width, stencil, Ic_w=None, tuning=None, fast_poisson=None):
        """``tuning``: dict with any of rhs_block, rows_per_lane, target_warps, min_piece (the
        launch shape of the triangular solves; missing or 0 = library default)."""
        Nj, Nf = circuit._Nj(), circuit._Nf()
        Rv, Cv, coef = coefficients(circuit, dt, stencil)
        Acsr = scipy.sparse.csr_matrix(A)
        Acsr.sort_indices()
        self._keep = dict(
            rowptr=np.ascontiguousarray(Acsr.indptr, np.int64),
            col=np.ascontiguousarray(Acsr.indices, np.int32),
            val=np.ascontiguousarray(Acsr.data, np.float64),
            Ic=np.ascontiguousarray(circuit._Ic(), np.float64),
            Ic_w=None if Ic_w is None else np.ascontiguousarray(Ic_w, np.float64),
            inv_c0=np.ascontiguousarray(1.0 / coef[0], np.float64),
            coef=np.ascontiguousarray(np.stack(coef[1:]), np.float64),
            Rv=np.ascontiguousarray(Rv, np.float64))
        k = self._keep
        ex = (ctypes.c_double * 4)(*(list(EXTRAP[stencil_width]) + [0.0] * (4 - len(EXTRAP[stencil_width]))))
        d = N.PlanDesc(Nj, Nf, W, stencil_width, N.ptr(k["rowptr"], ctypes.c_int64), N.ptr(k["col"], ctypes.c_int32),
                       N.ptr(k["val"]), N.ptr(k["Ic"]), N.ptr(k["inv_c0"]), N.ptr(k["coef"]), N.ptr(k["Rv"]), ex, dt,
                       N.ptr(k["Ic_w"]))
        tuning = dict(tuning or {})
        unknown = set(tuning) - set(TUNING_FIELDS)
        if unknown:
            raise ValueError(f"unknown tuning fields {sorted(unknown)}; expected {TUNING_FIELDS}")
        d.tuning = N.SolveTuning(*(int(tuning.get(f, 0)) for f in TUNING_FIELDS))
        self.tuning = {f: int(tuning.get(f, 0)) for f in TUNING_FIELDS}
        h = ctypes.c_void_p()
        N.check(N.lib().jja_plan_create(ctypes.byref(d), factor.handle, ctypes.byref(h)))
        self.handle = h
        self.Nj, self.Nf, self.W = Nj, Nf, W
        self.inv_c0 = k["inv_c0"]
        self.fast_poisson = False
        if fast_poisson is not None:
            mx, my, grid, kappa = fast_poisson
            self._keep["grid"] = grid
            N.check(N.lib().jja_plan_set_fast_poisson(h, int(mx), int(my), N.ptr(grid, ctypes.c_int32), float(kappa)))
            self.fast_poisson = True
        self.device_bytes = N.lib().jja_plan_device_bytes(h)

    def solve(self, b_dev, x_dev, stream=0):
        N.check(N.lib().jja_solve(self.handle, ctypes.c_void_p(b_dev), ctypes.c_void_p(x_dev), ctypes.c_void_p(stream)))

    def check(self):
        """Synchronise the device; raise JJAError if a wait of a dataflow sweep ran out of its
        bound since the last check (the steps since then are invalid)."""
        t = ctypes.c_int(0)
        N.check(N.lib().jja_plan_check(self.handle, ctypes.byref(t)))
        if t.value:
            raise N.JJAError(5, "a bounded wait of a dataflow or cooperative sweep ran out of its bound; "
                                "results are invalid")

    def eval_sin(self, x_dev, out_dev, n, stream=0):
        N.check(N.lib().jja_eval_sin(self.handle, ctypes.c_void_p(x_dev), ctypes.c_void_p(out_dev), int(n),
                                     ctypes.c_void_p(stream)))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.jja_plan_destroy(h)
            self.handle = None


def _coords(circuit):
    try:
        cx, cy = circuit.get_face_centroids()
        return np.asarray(cx, np.float64), np.asarray(cy, np.float64)
    except Exception:
        return None


MMD_MIN_WORK = 1 << 22     # "auto" picks minimum degree from this many face-problems (W x Nf) ...
MMD_MAX_FACES = 1 << 18    # ... on up to this many faces (its order comes from a host SuperLU run)


def resolve_ordering(ordering, W, n_faces):
    """The fill-reducing order "auto" stands for. When a step has a lot of work (W x Nf >= 2^22)
    the sweeps are FP64-bound, and minimum degree's factor has about 30 % fewer values than
    nested dissection's on 2D lattices (measured on GB300: 4 % less time per step for
    512 x SquareArray(128, 128)). With less work they are latency-bound, and nested dissection's
    tree has half the levels (64 x SquareArray(64, 64): minimum degree 54 % slower)."""
    if ordering == "auto":
        return "mmd" if W * n_faces >= MMD_MIN_WORK and n_faces <= MMD_MAX_FACES else "nd"
    return ordering


SMALL_STEP_FACES = 1 << 15   # W x Nf up to which "auto" factors with large leaves and strong amalgamation


def resolve_factor_shape(nd_leaf, relax, ordering, W, n_faces):
    """(nd_leaf, relax) that ``nd_leaf=None`` stands for. A step of few face-problems
    (W x Nf <= 2^15, nested dissection, default amalgamation) is bound by the elimination tree's
    depth: every level of each sweep is a chain of dependent memory round trips (about 3.5 us on
    GB300), and the flops are negligible. Such steps factor with nested-dissection leaves of 128
    faces and merge supernodes that add at most 256 zeros or 50 %: fewer, denser levels. Measured
    (W = 1, graph-replayed steps): SquareArray(10,10) 0.029 -> 0.014 ms/step (one dense
    supernode), SquareArray(128,128) 0.113 -> 0.081 ms; at 256x256 the larger factor costs more
    than the levels it saves (0.165 -> 0.205 ms), so larger steps keep leaves of 8."""
    if nd_leaf is not None:
        return nd_leaf, relax
    if ordering == "nd" and tuple(relax) == (-1, -1.0) and W * n_faces <= SMALL_STEP_FACES:
        return 128, (256, 0.5)
    return 8, relax


def fill_reducing_order(K, ordering, circuit=None):
    """(coords, perm) for HostFactor. "nd": the library's nested dissection on face centroids;
    "mmd": the multiple-minimum-degree column order scipy's SuperLU computes on A + A^T
    (less fill on 2D lattices, deeper elimination tree)."""
    if ordering == "nd":
        return (_coords(circuit) if circuit is not None else None), None
    if ordering == "mmd":
        import scipy.sparse.linalg
        lu = scipy.sparse.linalg.splu(K.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                                      options=dict(SymmetricMode=True))
        return None, np.argsort(lu.perm_c).astype(np.int32)
    raise ValueError(f"ordering must be 'nd' or 'mmd', not {ordering!r}")


def get_factor(circuit, dt, nd_leaf=8, ordering="nd", relax=(-1, -1.0)):
    A, K = face_matrix(circuit, dt)
    key = (_digest(K.indptr, K.indices, K.data), nd_leaf, ordering, tuple(relax))
    with _CACHE_LOCK:
        hit = _FACTORS.get(key)
        if hit is not None:
            _FACTORS.move_to_end(key)
            return hit[0], A, key
    coords, perm = fill_reducing_order(K, ordering, circuit)
    f = HostFactor(K, coords=coords, perm=perm, nd_leaf=nd_leaf, relax_zeros=relax[0], relax_frac=relax[1])
    with _CACHE_LOCK:
        _FACTORS[key] = (f, A)
        while len(_FACTORS) > MAX_FACTORS:
            _FACTORS.popitem(last=False)
    return f, A, key


def get_plan(circuit, dt, W, stencil_width, stencil, nd_leaf=None, ordering="auto", relax=(-1, -1.0), Ic_w=None,
             tuning=None, fast_poisson="auto"):
    """Device plan for W problems; ``Ic_w`` (Nj, W) gives each problem its own critical currents;
    ``ordering`` "nd", "mmd" or "auto" (see resolve_ordering); ``nd_leaf`` None: by the step's
    size (see resolve_factor_shape); ``tuning`` the launch shape of the triangular solves (see
    DevicePlan); ``fast_poisson``: solve with sine transforms when the face-space matrix allows it
    (fast_poisson_grid): True, False, or "auto" (W <= 8 and W x Nf <= 2^18 face-problems)."""
    ordering = resolve_ordering(ordering, W, circuit._Nf())
    nd_leaf, relax = resolve_factor_shape(nd_leaf, relax, ordering, W, circuit._Nf())
    fp = None
    if fast_poisson is True or (fast_poisson == "auto" and W <= FAST_POISSON_MAX_W
                                and W * circuit._Nf() <= FAST_POISSON_MAX_WORK):
        fp = fast_poisson_grid(circuit, face_matrix(circuit, dt)[1])
    factor, A, fkey = get_factor(circuit, dt, nd_leaf, ordering=ordering, relax=relax)
    Rv, Cv, coef = coefficients(circuit, dt, stencil)
    if Ic_w is not None:
        Ic_w = np.ascontiguousarray(np.broadcast_to(np.asarray(Ic_w, np.float64), (circuit._Nj(), W)))
    ic = np.asarray(circuit._Ic(), np.float64) if Ic_w is None else Ic_w
    tkey = tuple(int((tuning or {}).get(f, 0)) for f in TUNING_FIELDS)
    key = (fkey, W, stencil_width, Ic_w is None, tkey, fp is not None,
           _digest(ic, *coef, Rv, A.indptr, A.indices, A.data))
    with _CACHE_LOCK:
        p = _PLANS.get(key)
        if p is not None:
            _PLANS.move_to_end(key)
            return p
    p = DevicePlan(circuit, factor, A, W, dt, stencil_width, stencil, Ic_w=Ic_w, tuning=tuning, fast_poisson=fp)
    with _CACHE_LOCK:
        _PLANS[key] = p
        while len(_PLANS) > MAX_PLANS:
            _PLANS.popitem(last=False)
    return p


def clear_cache():
    with _CACHE_LOCK:
        _PLANS.clear()
        _FACTORS.clear()
