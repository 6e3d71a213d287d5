"""Static (stationary) problems on the GPU: pyjjasim's StaticProblem, StaticConfiguration and
NewtonIterInfo (static_problem.py:88-201, 389-1100) over the device Newton solver.

``StaticProblem.compute()`` runs the reference's Newton iteration ``static_compute``
(static_problem.py:1400-1515) with its stop rules, residuals and status in libjja_gb300
(``jja_static_newton``): every iteration refactors A (L + diag(1/q)) A^T, q = Ic cos(theta),
numerically on the GPU (supernodal LDL^T on a symbolic structure computed once per circuit) and
solves with it. ``approximate()`` is the London approximation (:1378-1395, ``jja_static_london``)
followed by the phase-zone change to zone 0 (:1145-1171). ``compute_many`` solves any number of
problems on one circuit in one batched iteration (every problem keeps its own iteration count);
AnnealingProblem uses it for its closing static refinement.

The phase-zone change needs an integral x with A x = z_new - z_old. The reference takes one from
a depth-first tree of the faces (embedded_graph.py:1041-1086); here a breadth-first tree of the
faces and the outer face gives another. Two integral solutions differ by 2 pi M^T k (k integral):
a gauge change that leaves currents, vortex configurations, the Newton iterates' residuals up to
rounding and every observable unchanged.
"""
import ctypes
import time

import numpy as np
import scipy.sparse
import scipy.sparse.csgraph
import scipy.sparse.linalg

from . import _native as N
from . import plan as P
from .problem import DefaultCPR

__all__ = ["StaticProblem", "StaticConfiguration", "NewtonIterInfo", "compute_many", "DEF_TOL",
           "DEF_NEWTON_MAXITER"]

DEF_TOL = 1e-10              # static_problem.py:25
DEF_NEWTON_MAXITER = 30      # static_problem.py:27


class NewtonIterInfo:
    """Record of one problem's Newton iteration (static_problem.py:88-201)."""

    def __init__(self, tol, maxiter, residuals, is_target, iterations, status, runtime):
        self.tol, self.maxiter = tol, maxiter
        self.error = np.asarray(residuals, np.double)
        self.is_target_n = np.asarray(is_target, int)
        self.iteration = iterations + 1          # number of recorded iterates
        self._status = int(status)
        self.has_converged = bool(self.error[iterations] < tol)
        self.runtime = runtime

    def get_max_iter(self):
        return self.maxiter

    def get_tol(self):
        return self.tol

    def get_status(self):
        return self._status

    def found_target_solution(self):
        return self.has_converged and bool(self.is_target_n[self._get_iteration()])

    def get_is_target_vortex_configuration(self):
        return self.is_target_n[:self.get_number_of_iterations() + 1]

    def get_number_of_iterations(self):
        return self._get_iteration()

    def get_residual(self):
        return self.error[:self.get_number_of_iterations() + 1]

    def get_runtime(self):
        return self.runtime

    def _get_iteration(self):
        return max(0, self.iteration - 1)

    def __str__(self):
        names = {0: " (converged)", 1: " (diverged)", 2: " (indeterminate; reached max_iter without converging or "
                                                         "diverging)"}
        return (f"newton iteration info: (tol={self.get_tol()}, maxiter={self.get_max_iter()})\n\t"
                f"status: {self.get_status()}{names.get(self.get_status(), '')}\n\t"
                f"number of iterations: {self.get_number_of_iterations()}\n\t"
                f"residual: {self.get_residual()}\n\truntime (in sec): {self.get_runtime()}")


def matrix_norm(B):
    """||B||_2 as the reference computes it (josephson_circuit.py:762-780): sqrt of the largest
    eigenvalue of B B^T."""
    B = scipy.sparse.csr_matrix(B).astype(np.double)
    if B.shape[0] == 1:
        return float(np.sqrt((B @ B.T).toarray()[0, 0]))
    return float(np.sqrt(scipy.sparse.linalg.eigsh(B @ B.T, 1, maxiter=1000, which="LA")[0][0]))


def integral_cycle_solve(circuit, b):
    """An integral x (..., Nj) with A x = b (..., Nf) for integral b (A: the cycle matrix, each
    junction on at most two faces): x is nonzero only on the edges of a breadth-first tree of the
    faces rooted at the outer face, each tree edge carrying the (signed) sum of b over the subtree
    behind it."""
    A = scipy.sparse.csc_matrix(circuit.get_cycle_matrix())
    Nf, Nj = A.shape
    b = np.asarray(b, np.double)
    shape = b.shape
    b = b.reshape(-1, Nf)
    outer = Nf
    # junction -> its faces (entries); junctions on one face connect it to the outer face
    nnz = np.diff(A.indptr)
    if np.any(nnz > 2):
        raise ValueError("a junction lies on more than two faces")
    fa = np.full(Nj, -1)
    fb = np.full(Nj, outer)
    va = np.zeros(Nj)
    vb = np.zeros(Nj)
    for j in np.flatnonzero(nnz >= 1):
        i0 = A.indptr[j]
        fa[j], va[j] = A.indices[i0], A.data[i0]
        if nnz[j] == 2:
            fb[j], vb[j] = A.indices[i0 + 1], A.data[i0 + 1]
    use = nnz >= 1
    js = np.flatnonzero(use)
    G = scipy.sparse.csr_matrix((np.ones(2 * len(js)), (np.r_[fa[js], fb[js]], np.r_[fb[js], fa[js]])),
                                shape=(Nf + 1, Nf + 1))
    order, pred = scipy.sparse.csgraph.breadth_first_order(G, outer, directed=False, return_predecessors=True)
    if len(order) != Nf + 1:
        raise ValueError("the faces and the outer face are not connected")
    # a junction between each pair of adjacent faces (the tree edge of a face to its predecessor)
    edge = {}
    for j in js:
        edge.setdefault((int(fa[j]), int(fb[j])), int(j))
        edge.setdefault((int(fb[j]), int(fa[j])), int(j))
    T = np.concatenate([b, np.zeros((b.shape[0], 1))], axis=1)    # subtree sums, outer face last
    x = np.zeros((b.shape[0], Nj))
    for f in order[:0:-1]:                                         # reverse BFS order, root excluded
        p = int(pred[f])
        j = edge[(int(f), p)]
        a_f = va[j] if fa[j] == f else vb[j]                       # A[f, j]
        x[:, j] = T[:, f] / a_f
        if p != outer:
            a_p = va[j] if fa[j] == p else vb[j]                   # A[p, j]
            T[:, p] -= a_p * x[:, j]
    return x.reshape(shape[:-1] + (Nj,))


def change_phase_zone(circuit, theta, z_old, z_new):
    """theta expressed in phase zone z_new (static_problem.py:1145-1171)."""
    dz = np.broadcast_to(np.asarray(z_new) - np.asarray(z_old), (circuit._Nf(),))
    if np.all(dz == 0):
        return theta
    return theta + integral_cycle_solve(circuit, dz.astype(np.double)) * 2.0 * np.pi


class StaticPlan:
    """Device plan of the static solver for W problems on one circuit (owned C object)."""

    def __init__(self, circuit, W):
        A = scipy.sparse.csr_matrix(circuit.get_cycle_matrix()).astype(np.double)
        A.sort_indices()
        M = scipy.sparse.csr_matrix(circuit.get_cut_matrix()).astype(np.double)
        M.sort_indices()
        Nj, Nf, Nn = A.shape[1], A.shape[0], M.shape[0]
        L = scipy.sparse.csr_matrix(circuit._L()).astype(np.double)
        L.eliminate_zeros()
        L.sort_indices()
        has_L = L.nnz > 0
        # symbolic structure: the pattern of A (L + D) A^T for a diagonal D
        Kpat = (A @ (L + scipy.sparse.identity(Nj)) @ A.T).tocsc()
        Kpat.sum_duplicates()
        Kpat.sort_indices()
        self.factor = P.HostFactor(Kpat, coords=P._coords(circuit))
        KL = None
        if has_L:
            KL = (A @ L @ A.T).tocsc()
            KL.sum_duplicates()
            KL.sort_indices()
        self.A_norm, self.M_norm = matrix_norm(A), matrix_norm(M)
        k = self._keep = dict(
            a_rp=np.ascontiguousarray(A.indptr, np.int64), a_ci=np.ascontiguousarray(A.indices, np.int32),
            a_v=np.ascontiguousarray(A.data, np.float64),
            m_rp=np.ascontiguousarray(M.indptr, np.int64), m_ci=np.ascontiguousarray(M.indices, np.int32),
            m_v=np.ascontiguousarray(M.data, np.float64),
            l_rp=np.ascontiguousarray(L.indptr, np.int64) if has_L else None,
            l_ci=np.ascontiguousarray(L.indices, np.int32) if has_L else None,
            l_v=np.ascontiguousarray(L.data, np.float64) if has_L else None,
            kl_cp=np.ascontiguousarray(KL.indptr, np.int64) if has_L else None,
            kl_ri=np.ascontiguousarray(KL.indices, np.int32) if has_L else None,
            kl_v=np.ascontiguousarray(KL.data, np.float64) if has_L else None,
            Ic=np.ascontiguousarray(np.broadcast_to(circuit._Ic(), (Nj,)), np.float64))
        I64, I32 = ctypes.c_int64, ctypes.c_int32
        d = N.StaticDesc(Nj, Nf, Nn, W, N.ptr(k["a_rp"], I64), N.ptr(k["a_ci"], I32), N.ptr(k["a_v"]),
                         N.ptr(k["m_rp"], I64), N.ptr(k["m_ci"], I32), N.ptr(k["m_v"]),
                         N.ptr(k["l_rp"], I64), N.ptr(k["l_ci"], I32), N.ptr(k["l_v"]),
                         N.ptr(k["kl_cp"], I64), N.ptr(k["kl_ri"], I32), N.ptr(k["kl_v"]),
                         N.ptr(k["Ic"]), self.A_norm, self.M_norm)
        h = ctypes.c_void_p()
        N.check(N.lib().jja_static_create(ctypes.byref(d), self.factor.handle, ctypes.byref(h)))
        self.handle = h
        self.Nj, self.Nf, self.Nn, self.W = Nj, Nf, Nn, W
        self.device_bytes = N.lib().jja_static_device_bytes(h)

    def _dev(self, a, dtype):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()

    def solve(self, iq, b):
        """(A (L + diag(iq_w)) A^T)^-1 b_w per problem; iq (W, Nj), b (W, Nf); returns (x, pivot errors)."""
        import torch
        iq_d, b_d = self._dev(iq, np.float64), self._dev(b, np.float64)
        x = torch.empty_like(b_d)
        err = (ctypes.c_int * self.W)()
        N.check(N.lib().jja_static_solve(self.handle, ctypes.c_void_p(iq_d.data_ptr()), ctypes.c_void_p(b_d.data_ptr()),
                                         ctypes.c_void_p(x.data_ptr()), err, None))
        torch.cuda.synchronize()
        return x.cpu().numpy(), np.array(err[:], dtype=int)

    def london(self, Is, f, n):
        """London approximation (W, Nj) in phase zone n: Is (W, Nj), f (W, Nf), n (W, Nf)."""
        import torch
        Is_d, f_d, n_d = self._dev(Is, np.float64), self._dev(f, np.float64), self._dev(n, np.int32)
        th = torch.empty_like(Is_d)
        N.check(N.lib().jja_static_london(self.handle, ctypes.c_void_p(Is_d.data_ptr()), ctypes.c_void_p(f_d.data_ptr()),
                                          ctypes.c_void_p(n_d.data_ptr()), ctypes.c_void_p(th.data_ptr()), None))
        torch.cuda.synchronize()
        return th.cpu().numpy()

    def newton(self, theta0, Is, f, n, tol=DEF_TOL, maxiter=DEF_NEWTON_MAXITER, stop_as_residual_increases=True,
               stop_if_not_target_n=False):
        """Device static_compute for every problem: returns theta (W, Nj), status, iterations,
        residuals (W, maxiter + 1), is_target (W, maxiter + 1)."""
        import torch
        th = self._dev(theta0, np.float64)
        Is_d, f_d, n_d = self._dev(Is, np.float64), self._dev(f, np.float64), self._dev(n, np.int32)
        W, R = self.W, int(maxiter) + 1
        status, iters = (ctypes.c_int * W)(), (ctypes.c_int * W)()
        res = np.zeros((W, R))
        tgt = np.zeros((W, R), np.int32)
        a = N.NewtonArgs(th.data_ptr(), Is_d.data_ptr(), f_d.data_ptr(), n_d.data_ptr(), float(tol), int(maxiter),
                         int(bool(stop_as_residual_increases)), int(bool(stop_if_not_target_n)))
        r = N.NewtonResult(status, iters, N.ptr(res), tgt.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        N.check(N.lib().jja_static_newton(self.handle, ctypes.byref(a), ctypes.byref(r), None))
        torch.cuda.synchronize()
        return th.cpu().numpy(), np.array(status[:]), np.array(iters[:]), res, tgt

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.jja_static_destroy(h)
            self.handle = None


_PLANS = {}
MAX_PLANS = 4


def get_static_plan(circuit, W):
    """The device static plan of a circuit for W problems, cached by the circuit's content."""
    from .backend import _torch
    _torch()
    Lm = scipy.sparse.csr_matrix(circuit._L())
    key = (P._digest(circuit.get_cycle_matrix().toarray() if circuit._Nf() * circuit._Nj() < 4e6 else
                     scipy.sparse.csr_matrix(circuit.get_cycle_matrix()).indices,
                     np.broadcast_to(circuit._Ic(), (circuit._Nj(),)), Lm.indptr, Lm.indices, Lm.data,
                     scipy.sparse.csr_matrix(circuit.get_cut_matrix()).indices), W)
    p = _PLANS.get(key)
    if p is None:
        p = StaticPlan(circuit, W)
        _PLANS[key] = p
        while len(_PLANS) > MAX_PLANS:
            _PLANS.pop(next(iter(_PLANS)))
    return p


class StaticProblem:
    """A static Josephson junction array problem (static_problem.py:389-812); ``compute()`` and
    ``approximate()`` run on the GPU."""

    def __init__(self, circuit, current_sources=0.0, external_flux=0.0, vortex_configuration=0,
                 current_phase_relation=None):
        self.circuit = circuit
        self.current_sources = np.atleast_1d(current_sources)
        self.external_flux = np.atleast_1d(external_flux)
        self.vortex_configuration = np.atleast_1d(vortex_configuration)
        self.current_phase_relation = DefaultCPR() if current_phase_relation is None else current_phase_relation

    def get_circuit(self):
        return self.circuit

    def get_current_sources(self):
        return self.current_sources

    def get_external_flux(self):
        return self.external_flux

    def get_vortex_configuration(self):
        return self.vortex_configuration

    def get_current_phase_relation(self):
        return self.current_phase_relation

    def get_phase_zone(self):
        return 0

    def _Is(self):
        return self.current_sources

    def _f(self):
        return self.external_flux

    def _nt(self):
        return self.vortex_configuration

    def _cp(self, Ic, theta):
        return self.current_phase_relation.eval(Ic, theta)

    def approximate(self):
        """London approximation in phase zone 0 (static_problem.py:550-557)."""
        return approximate_many([self])[0]

    def compute(self, initial_guess=None, tol=DEF_TOL, maxiter=DEF_NEWTON_MAXITER, stop_as_residual_increases=True,
                stop_if_not_target_n=False):
        """Newton iteration from ``initial_guess`` (default: approximate()); returns
        (StaticConfiguration, status, NewtonIterInfo) like the reference (static_problem.py:559-607)."""
        return compute_many([self], None if initial_guess is None else [initial_guess], tol=tol, maxiter=maxiter,
                            stop_as_residual_increases=stop_as_residual_increases,
                            stop_if_not_target_n=stop_if_not_target_n)[0]


class StaticConfiguration:
    """theta of a static problem and the quantities it defines (static_problem.py:815-1100)."""

    def __init__(self, problem, theta):
        self.problem = problem
        self.theta = np.array(theta, dtype=np.double)
        if self.theta.shape != (problem.get_circuit()._Nj(),):
            raise ValueError("theta must be of shape (Nj,)")

    def get_circuit(self):
        return self.problem.get_circuit()

    def get_problem(self):
        return self.problem

    def _th(self):
        return self.theta

    def get_theta(self):
        return self.theta

    def get_phase(self):
        M = self.get_circuit().get_cut_matrix()
        return self.get_circuit().Msq_solve(M @ self.theta)

    def get_vortex_configuration(self):
        A = self.get_circuit().get_cycle_matrix()
        return -(A @ np.round(self.theta / (2.0 * np.pi))).astype(int)

    def get_current(self):
        return self.problem._cp(self.get_circuit()._Ic(), self.theta)

    def get_cycle_current(self):
        A = self.get_circuit().get_cycle_matrix()
        return self.get_circuit().Asq_solve(A @ (self.get_current() - self.problem.current_sources))

    def get_flux(self):
        A = self.get_circuit().get_cycle_matrix()
        return self.problem.external_flux + A @ (self.get_circuit()._L() @ self.get_current()) / (2 * np.pi)

    def satisfies_target_vortices(self):
        return bool(np.all(self.get_vortex_configuration() == self.problem._nt()))


def _stack(problems):
    c = problems[0].get_circuit()
    for p in problems:
        if p.get_circuit() is not c:
            raise ValueError("the problems of one batch must share their circuit")
        if type(p.get_current_phase_relation()).__name__ != "DefaultCPR":
            raise NotImplementedError("the GPU static solver evaluates the default current-phase relation only")
    Nj, Nf = c._Nj(), c._Nf()
    Is = np.stack([np.broadcast_to(np.asarray(p._Is(), np.double), (Nj,)) for p in problems])
    f = np.stack([np.broadcast_to(np.asarray(p._f(), np.double), (Nf,)) for p in problems])
    n = np.stack([np.broadcast_to(np.asarray(p._nt()), (Nf,)).astype(np.int32) for p in problems])
    return c, Is, f, n


def approximate_many(problems):
    """StaticProblem.approximate() of problems on one circuit, in one batched device solve."""
    c, Is, f, n = _stack(problems)
    th = get_static_plan(c, len(problems)).london(Is, f, n)
    return [StaticConfiguration(p, change_phase_zone(c, th[w], n[w], 0)) for w, p in enumerate(problems)]


def compute_many(problems, initial_guesses=None, tol=DEF_TOL, maxiter=DEF_NEWTON_MAXITER,
                 stop_as_residual_increases=True, stop_if_not_target_n=False):
    """StaticProblem.compute() of problems on one circuit, batched: one device Newton iteration
    for all of them (each stops by the reference's rules on its own). Returns a list of
    (StaticConfiguration, status, NewtonIterInfo)."""
    t0 = time.perf_counter()
    c, Is, f, n = _stack(problems)
    W = len(problems)
    initial_guesses = [None] * W if initial_guesses is None else list(initial_guesses)
    approx = approximate_many(problems) if any(g is None for g in initial_guesses) else None
    guesses = [approx[w].get_theta() if g is None else (g._th() if isinstance(g, StaticConfiguration) else g)
               for w, g in enumerate(initial_guesses)]
    th0 = np.stack([np.asarray(g, np.double) for g in guesses])
    th, status, iters, res, tgt = get_static_plan(c, W).newton(th0, Is, f, n, tol, maxiter, stop_as_residual_increases,
                                                               stop_if_not_target_n)
    rt = time.perf_counter() - t0
    return [(StaticConfiguration(p, th[w]), int(status[w]),
             NewtonIterInfo(tol, maxiter, res[w], tgt[w], int(iters[w]), int(status[w]), rt))
            for w, p in enumerate(problems)]
