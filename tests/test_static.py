"""Static (Newton) problems: the oracle against the reference's own StaticProblem.compute()
(tests/golden/s*.npz, a1_*.npz), and the GPU solver against both.

Fixtures: four problems the reference's iteration solves (square with a vortex, honeycomb with
inductance, triangular with disordered Ic, square with inductance and a vortex) and two it gives
up on (bias above the critical current; a poor initial guess), each with the reference's initial
guess (approximate()), solution, status, iteration count, residual history and target flags.
Phases are compared modulo 2 pi: the reference picks its phase-zone representative through a
depth-first tree of the faces, this package through a breadth-first one; the two differ by
2 pi M^T k, a gauge change that moves no current, vortex or residual.
"""
import glob
import os

import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg

import golden_cases as gc
from oracle import static_oracle as SO
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray
from pyjjasim_gb300.static import change_phase_zone, integral_cycle_solve

CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(gc.GOLDEN, "s*.npz")))


def _case(name):
    z = gc.load(name)
    kw = {"tol": float(z["param_tol"]), "maxiter": int(z["param_maxiter"])} if "param_tol" in z else {}
    return z, gc.circuit(z), kw


def _same_mod_2pi(a, b, atol):
    d = (np.asarray(a) - np.asarray(b)) / (2 * np.pi)
    return float(np.abs(d - np.round(d)).max()) <= atol / (2 * np.pi)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    z, c, kw = _case(name)
    th, st, res, tgt = SO.static_compute(c.get_cycle_matrix(), c.get_cut_matrix(), c._L(), c._Ic(), z["theta0"],
                                         z["in_Is"], z["in_f"], z["in_n"], **kw)
    assert st == int(z["status"]) and len(res) - 1 == int(z["iterations"])
    np.testing.assert_allclose(res, z["residuals"], rtol=1e-6, atol=1e-12)
    assert np.array_equal(tgt, z["is_target"])
    assert _same_mod_2pi(th, z["theta"], 1e-11)


@pytest.mark.parametrize("make", [lambda: SquareArray(9, 7), lambda: HoneycombArray(4, 5),
                                  lambda: TriangularArray(6, 5)])
def test_integral_cycle_solve(make):
    c = make()
    b = np.random.default_rng(1).integers(-4, 5, (3, c.face_count())).astype(float)
    x = integral_cycle_solve(c, b)
    assert np.array_equal(x, np.round(x))
    np.testing.assert_array_equal((c.get_cycle_matrix() @ x.T).T, b)


@pytest.mark.parametrize("name", [n for n in CASES if not gc.load(n)["guess_given"]])
def test_london_guess_matches_reference_up_to_gauge(name):
    z, c, _ = _case(name)
    A = c.get_cycle_matrix()
    th = change_phase_zone(c, SO.london_approximation(A, c._L(), c._Ic(), z["in_f"], z["in_n"], z["in_Is"]),
                           z["in_n"], 0)
    k = (th - z["theta0"]) / (2 * np.pi)
    assert np.abs(k - np.round(k)).max() < 1e-9
    assert np.abs(A @ np.round(k)).max() == 0          # a gauge change: A k = 0


# ------------------------------------------------------------------------------- GPU -------
@pytest.mark.gpu
@pytest.mark.parametrize("make", [lambda: SquareArray(23, 17), lambda: HoneycombArray(7, 6),
                                  lambda: TriangularArray(11, 9), lambda: SquareArray(70, 64)])
@pytest.mark.parametrize("L", [0.0, 0.3])
def test_device_factorisation_solves_indefinite_systems(make, L):
    """The device LDL^T (no pivoting) of A (L + diag(iq)) A^T for three problems, one with a
    few negative iq (cos(theta) < 0 at some junctions), against scipy's sparse LU."""
    from pyjjasim_gb300.static import get_static_plan
    c = make()
    c.set_inductance(L)
    W = 3
    rng = np.random.default_rng(7)
    q = rng.uniform(0.4, 1.5, (W, c.junction_count()))
    q[2, rng.choice(c.junction_count(), 3, replace=False)] *= -1.0
    iq = 1.0 / q
    b = rng.standard_normal((W, c.face_count()))
    x, err = get_static_plan(c, W).solve(iq, b)
    assert not err.any()
    A = scipy.sparse.csr_matrix(c.get_cycle_matrix()).astype(float)
    for w in range(W):
        K = (A @ (scipy.sparse.csr_matrix(c._L()) + scipy.sparse.diags(iq[w])) @ A.T).tocsc()
        ref = scipy.sparse.linalg.spsolve(K, b[w])
        assert np.abs(x[w] - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_device_newton_matches_reference(name):
    """From the reference's initial guess: same status, iteration count, target flags; residual
    history within 1e-6 relative; phases within 1e-9 modulo 2 pi."""
    from pyjjasim_gb300.static import StaticProblem
    z, c, kw = _case(name)
    p = StaticProblem(c, current_sources=z["in_Is"], external_flux=z["in_f"], vortex_configuration=z["in_n"])
    cfg, status, info = p.compute(initial_guess=z["theta0"], **kw)
    assert status == int(z["status"]) and info.get_number_of_iterations() == int(z["iterations"])
    np.testing.assert_allclose(info.get_residual(), z["residuals"], rtol=1e-6, atol=1e-12)
    assert np.array_equal(info.get_is_target_vortex_configuration(), z["is_target"])
    if status == 0:
        assert _same_mod_2pi(cfg.get_theta(), z["theta"], 1e-9)
        np.testing.assert_allclose(cfg.get_current(), z["current"], atol=1e-9)
        assert np.array_equal(cfg.get_vortex_configuration(), z["vortex"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in CASES if not gc.load(n)["guess_given"]])
def test_device_compute_from_its_own_guess(name):
    """compute() with the device London approximation as the guess (the reference's default
    path): the guess equals the reference's up to a gauge change, the outcome equals it."""
    from pyjjasim_gb300.static import StaticProblem
    z, c, kw = _case(name)
    p = StaticProblem(c, current_sources=z["in_Is"], external_flux=z["in_f"], vortex_configuration=z["in_n"])
    k = (p.approximate().get_theta() - z["theta0"]) / (2 * np.pi)
    assert np.abs(k - np.round(k)).max() < 1e-9 and np.abs(c.get_cycle_matrix() @ np.round(k)).max() == 0
    cfg, status, info = p.compute(**kw)
    assert status == int(z["status"]) and info.get_number_of_iterations() == int(z["iterations"])
    if status == 0:
        assert _same_mod_2pi(cfg.get_theta(), z["theta"], 1e-9)
        assert np.array_equal(cfg.get_vortex_configuration(), z["vortex"])


@pytest.mark.gpu
def test_batched_problems_match_the_oracle_one_by_one():
    """Twelve problems on one 40x36 array (different biases, fluxes, vortices) in one batched
    device iteration, each against the oracle run alone; they stop after different counts.
    Converged ones agree in every residual and in theta; diverging ones in status, iteration
    count and starting residual."""
    from pyjjasim_gb300.static import StaticProblem, compute_many
    c = SquareArray(40, 36)
    c.set_inductance(0.1)
    # (bias, current angle, flux, target vortex face or -1): the oracle converges on the first six
    # after 0, 2, 2, 7, 4 and 2 iterations and gives up on the others
    spec = [(0.0, 0.0, 0.0, -1), (0.3, 0.0, 0.0, -1), (0.2, 0.0, 0.0, -1), (0.05, 0.0, 0.02, -1),
            (0.05, 1.8, 0.02, -1), (0.1, 0.0, 0.0, -1), (0.15, 0.3, 0.05, -1), (0.35, 0.9, 0.02, 700),
            (0.25, 0.6, 0.08, -1), (0.45, 1.2, 0.05, -1), (0.15, 2.1, 0.05, 700), (0.55, 3.3, 0.08, 700)]
    probs = []
    for bias, angle, f, face in spec:
        n = np.zeros(c.face_count(), int)
        if face >= 0:
            n[face] = 1
        probs.append(StaticProblem(c, current_sources=bias * c.current_base(angle), external_flux=f,
                                   vortex_configuration=n))
    out = compute_many(probs)
    A, M = c.get_cycle_matrix(), c.get_cut_matrix()
    guesses = [p.approximate().get_theta() for p in probs]
    iters = set()
    for p, g, (cfg, status, info) in zip(probs, guesses, out):
        th, st, res, tgt = SO.static_compute(A, M, c._L(), c._Ic(), g, p._Is(), p._f(), p._nt())
        assert status == st and info.get_number_of_iterations() == len(res) - 1
        if st == 0:
            np.testing.assert_allclose(info.get_residual(), res, rtol=1e-6, atol=1e-12)
            assert _same_mod_2pi(cfg.get_theta(), th, 1e-9)
        else:
            # a diverging iteration (residual near 0.5, q = Ic cos(theta) near zero) amplifies
            # rounding from one iterate to the next; the stop rule and status still agree
            np.testing.assert_allclose(info.get_residual()[:1], res[:1], rtol=1e-9)
        iters.add(info.get_number_of_iterations())
    assert len(iters) > 1


@pytest.mark.gpu
def test_annealing_compute_returns_the_reference_triple():
    """AnnealingProblem.compute() with the reference's noise replayed: the temperature profiles,
    the statuses of the closing static refinement and the static configurations of the
    reference's own run (a1 fixture)."""
    from pyjjasim_gb300.annealing import AnnealingProblem
    z = gc.load("a1_square6x5_anneal")
    c = gc.circuit(z)
    params = {k: z["param_" + k].item() for k in ("time_step", "interval_steps", "interval_count", "problem_count",
                                                  "external_flux", "vortex_mobility", "start_T", "T_factor")}
    np.random.seed(int(z["seed"]))
    status, configs, profiles = AnnealingProblem(c, **params).compute(noise="numpy")
    np.testing.assert_allclose(profiles, z["temperature_profiles"], rtol=1e-13, atol=0)
    np.testing.assert_array_equal(status, z["status"])
    for w, cfg in enumerate(configs):
        if status[w] == 0:
            assert _same_mod_2pi(cfg.get_theta(), z["static_theta"][:, w], 1e-9)
            assert np.array_equal(cfg.get_vortex_configuration(), z["final_vortex"][:, w])
