"""CPU oracle for the static (Newton) problem (TEST INFRASTRUCTURE ONLY).

The checker of the static row, never the product: only tests/ import it. Restates in numpy/scipy
FP64 the reference's
* ``static_compute`` (pyjjasim static_problem.py:1400-1515): Newton iteration on
  theta with q = Ic cos(theta) (|q| < 0.1 tol set to 0.1 tol), S = L + diag(1/q),
  y = (I - Is)/q, j = (A S A^T)^-1 (A (theta - y - L Is) + 2 pi (f - z)), theta -= y + A^T j / q
  (theta += 1e10 when j is not finite); the stop rules and the NewtonIterInfo status
  (:88-201);
* ``get_kirchhoff_error`` / ``get_winding_error`` (:1108-1130), with ||A||_2 and ||M||_2 from
  the largest eigenvalue of A A^T and M M^T (josephson_circuit.py:762-780);
* ``london_approximation`` (:1378-1395).
The matrices are factorised with scipy's SuperLU (``factorized``), as the reference does.
Pinned: tests/test_static.py checks this oracle against fixtures of the reference's own
StaticProblem.compute() (tests/golden/s*.npz).
"""
import numpy as np
import scipy.linalg
import scipy.sparse
import scipy.sparse.linalg


def matrix_norm(B):
    """||B||_2 as the reference computes it: sqrt of the largest eigenvalue of B B^T."""
    B = scipy.sparse.csr_matrix(B).astype(np.double)
    if B.shape[0] == 1:
        return float(np.sqrt((B @ B.T).toarray()[0, 0]))
    return float(np.sqrt(scipy.sparse.linalg.eigsh(B @ B.T, 1, maxiter=1000, which="LA")[0][0]))


def kirchhoff_error(M, M_norm, I, Is, Is_norm):
    b = M @ (I - Is)
    normalizer = M_norm * (Is_norm + scipy.linalg.norm(I))
    return np.finfo(float).eps if abs(normalizer) < 1e-20 else scipy.linalg.norm(b) / normalizer


def winding_error(A, A_norm, L, th, I, df):
    def norm(x):
        return scipy.linalg.norm(x) / np.sqrt(len(x))
    LI = L @ I
    normalizer = A_norm * (norm(th) + norm(LI)) + norm(df)
    return np.finfo(float).eps if abs(normalizer) < 1e-20 else norm(df + A @ (th + LI)) / normalizer


def london_approximation(A, L, Ic, f, n, Is):
    """theta of the London (linearised) approximation in phase zone n (static_problem.py:1378-1395)."""
    Nf = A.shape[0]
    iIc = np.array(Ic, dtype=np.double, copy=True)
    big = np.abs(iIc) > 1e-12
    iIc[big] = 1.0 / iIc[big]
    D = scipy.sparse.diags(iIc)
    K = (A @ (D + L) @ A.T).tocsc()
    df = 2 * np.pi * np.broadcast_to(n - f, (Nf,))
    Isc = np.broadcast_to(Is, (A.shape[1],))
    return D @ (A.T @ scipy.sparse.linalg.factorized(K)(df - A @ (D + L) @ Isc) + Isc)


def static_compute(A, M, L, Ic, theta0, Is, f, n, z=0, tol=1e-10, maxiter=30, stop_as_residual_increases=True,
                   stop_if_not_target_n=False, A_norm=None, M_norm=None):
    """Returns (theta, status, residuals, is_target) of the reference's Newton iteration."""
    A = scipy.sparse.csr_matrix(A).astype(np.double)
    M = scipy.sparse.csr_matrix(M).astype(np.double)
    L = scipy.sparse.csr_matrix(L)
    Nj, Nf = A.shape[1], A.shape[0]
    A_norm = matrix_norm(A) if A_norm is None else A_norm
    M_norm = matrix_norm(M) if M_norm is None else M_norm
    Ic = np.broadcast_to(Ic, (Nj,))
    Is = np.ones(Nj) * Is if np.array(Is).size == 1 else np.asarray(Is, np.double)
    f = np.ones(Nf) * f if np.array(f).size == 1 else np.asarray(f, np.double)
    n = np.ones(Nf, dtype=int) * n if np.array(n).size == 1 else np.asarray(n)
    df = 2 * np.pi * (f - z)
    theta = np.array(theta0, dtype=np.double, copy=True)
    I = Ic * np.sin(theta)
    LIs = L @ Is
    Is_norm = scipy.linalg.norm(Is)
    errors, targets = [], []

    def record():
        e = max(kirchhoff_error(M, M_norm, I, Is, Is_norm), winding_error(A, A_norm, L, theta, I, df))
        t = bool(np.all(A @ (np.round(theta / (2 * np.pi))).astype(int) == z - n))
        errors.append(e)
        targets.append(t)
        return e, t

    error, is_target = record()
    prev_error, iteration = np.inf, 0
    while not (error < tol or (error > 0.5 and iteration > 5) or (stop_if_not_target_n and is_target)
               or (stop_as_residual_increases and error > prev_error) or iteration >= maxiter):
        q = Ic * np.cos(theta)
        q[np.abs(q) < 0.1 * tol] = 0.1 * tol
        S = L + scipy.sparse.diags(1 / q, 0)
        y = (I - Is) / q
        j = scipy.sparse.linalg.factorized((A @ S @ A.T).tocsc())(A @ (theta - y - LIs) + df)
        if np.any(np.isnan(j)) or np.any(np.isinf(j)):
            theta += 10 ** 10
        else:
            theta -= y + (A.T @ j) / q
        I = Ic * np.sin(theta)
        error, is_target = record()
        if iteration >= 3:
            prev_error = errors[iteration - 3]
        iteration += 1
    last = max(0, len(errors) - 1)
    found = errors[last] < tol and targets[last]
    status = int(not found) + 2 * int(iteration >= maxiter)
    return theta, status, np.array(errors), np.array(targets, dtype=int)
