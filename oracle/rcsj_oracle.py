"""CPU oracle for the RCSJ time-evolution hot path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only tests/, the smoke check in
__graft_entry__.py and the CPU-baseline leg of bench.py may import it. The product
path (package ``pyjjasim_gb300``) never imports anything under ``oracle/``.

It restates, in plain numpy/scipy FP64, the reference's per-step update
``time_evolution_core`` (pyjjasim time_evolution.py:461-582) and the voltage
post-processing of ``time_evolution`` (time_evolution.py:411-458), reading inputs
through the same duck-typed problem interface the reference uses
(``_Is/_T/_Vs/_f``, ``_*_is_timedep``, ``stencil``, ``config_at_minus_*``,
circuit ``get_cycle_matrix/_Ic/_R/_C/_L``). The face-space solve uses the same
library factorisation as the reference (``scipy.sparse.linalg.factorized``,
time_evolution.py:505-506), so on identical inputs the oracle reproduces the
reference bit for bit at T=0 and, given the same ``np.random`` seed, at T>0.

Pinned: tests/test_oracle_golden.py checks this oracle against golden vectors that
tests/golden/make_golden.py produced by running the reference's own ``compute()``.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg


def stencil(width):
    """Backward-difference stencils (first, second derivative); time_evolution.py:401-408."""
    if width == 3:
        return (1.0, -1.0, 0.0), (1.0, -2.0, 1.0)
    if width == 4:
        return (1.5, -2.0, 0.5, 0.0), (2.0, -5.0, 4.0, -1.0)
    if width == 5:
        return (11.0 / 6, -3.0, 1.5, -1.0 / 3, 0.0), (35.0 / 12, -26.0 / 3, 9.5, -14.0 / 3, 11.0 / 12)
    raise ValueError(f"stencil width must be 3, 4 or 5 (equals {width})")


# Extrapolation of the CPR argument from the phase history (time_evolution.py:547-553):
# width 3: 2*th1 - th2; width 4: 3*th1 - 3*th2 + th3; width 5: 4*th1 - 6*th2 + 4*th3 - th4.
EXTRAP = {3: (2.0, -1.0), 4: (3.0, -3.0, 1.0), 5: (4.0, -6.0, 4.0, -1.0)}


class NumpyGlobalNoise:
    """Standard-normal draws in the reference's ``np.random`` call order (time_evolution.py:533-538).

    For more than 500 junctions a fresh ``randn(Nj, W)`` is drawn only on steps with
    i % 3 == 0; the other steps reuse the previous draw with rows permuted by
    ``np.random.permutation(Nj)``. Otherwise a fresh draw is made every step.
    """

    def __init__(self, Nj, W):
        self.Nj, self.W, self.prev = Nj, W, None

    def __call__(self, i):
        if self.Nj > 500:
            if i % 3 == 0:
                self.prev = np.random.randn(self.Nj, self.W)
            else:
                self.prev = self.prev[np.random.permutation(self.Nj), :]
        else:
            self.prev = np.random.randn(self.Nj, self.W)
        return self.prev


def evolve(problem, th_store_mask, I_store_mask, noise=None, on_step=None, factorize=None):
    """Restatement of time_evolution_core (time_evolution.py:461-582).

    Returns (th_out, I_out) of shape (Nj, W, sum(mask) + width - 1); slots
    0..width-2 hold the initial conditions (theta and cp(theta)), oldest first.
    ``noise``: callable i -> (Nj, W) standard normals; default NumpyGlobalNoise.
    ``on_step``: optional callable(i) run after step i (used to time the loop).
    ``factorize``: optional callable K -> solve function replacing the reference's
    ``scipy.sparse.linalg.factorized`` (a different fill-reducing order of the same LU gives the
    same algorithm with another rounding: it measures how far rounding alone moves a trajectory).
    """
    c = problem.get_circuit()
    Nj, W, dt = c._Nj(), problem.get_problem_count(), problem._dt()
    width = problem.stencil_width
    s1, s2 = problem.stencil
    A = c.get_cycle_matrix()
    Rv = 1.0 / (dt * c._R()[:, None])                       # :472
    Cv = c._C()[:, None] / dt ** 2                          # :473
    # coefficient of theta at lag k in the stencil combination (:477-478, 489, 495, 501)
    coef = [s1[k] * Rv + s2[k] * Cv for k in range(width)]
    c0 = coef[0]
    Cnext = Cv + Rv                                         # :476 (used for the matrix for every width)
    Ic = c._Ic()[:, None]

    hist = [problem.config_at_minus_1.copy(), problem.config_at_minus_2.copy()]
    if width >= 4:
        hist.append(problem.config_at_minus_3.copy())
    if width >= 5:
        hist.append(problem.config_at_minus_4.copy())
    n_init = width - 1
    th_out = np.zeros((Nj, W, int(np.sum(th_store_mask)) + n_init))
    I_out = np.zeros((Nj, W, int(np.sum(I_store_mask)) + n_init))
    for lag, th in enumerate(hist):                          # slot width-2-lag holds t = -1-lag
        th_out[:, :, n_init - 1 - lag] = th
        I_out[:, :, n_init - 1 - lag] = problem._cp(th)

    K = A @ (c._L() + scipy.sparse.diags(1.0 / Cnext[:, 0], 0)) @ A.T   # :504-505
    solve = (factorize or scipy.sparse.linalg.factorized)(K)           # :506
    theta_s = np.zeros((Nj, W))

    Is, T, Vs, f = problem._Is(0), problem._T(0), problem._Vs(0), problem._f(0)
    T_zero = (not problem._T_is_timedep) and np.allclose(T, 0)          # :512-519
    Is_zero = (not problem._Is_is_timedep) and np.allclose(Is, 0)
    Vs_zero = (not problem._Vs_is_timedep) and np.allclose(Vs, 0)
    f_zero = (not problem._f_is_timedep) and np.allclose(f, 0)
    if noise is None and not T_zero:
        noise = NumpyGlobalNoise(Nj, W)
    ex = EXTRAP[width]
    fluct = 0.0
    k_th = k_I = n_init
    for i in range(problem._Nt()):
        if problem._T_is_timedep:
            T = problem._T(i)
        if problem._Is_is_timedep:
            Is = problem._Is(i)
        if problem._Vs_is_timedep:
            Vs = problem._Vs(i)
        if problem._f_is_timedep:
            f = problem._f(i)
        if not T_zero:
            fluct = np.sqrt(2.0 * T * Rv) * noise(i)                   # :537
        # hist[0] = theta at step i-1, hist[1] at i-2, ...
        arg = sum(e * h for e, h in zip(ex, hist))
        X = problem._cp(arg)
        for k in range(1, width):
            X = X + coef[k] * hist[k - 1]
        x = (fluct + X) if Is_zero else (fluct - Is + X)               # :555-558
        rhs = x / c0 if Vs_zero else x / c0 - theta_s
        b = A @ rhs
        if not f_zero:
            b = b - 2 * np.pi * f
        y = A.T @ solve(b)                                             # :560-569
        th_next = (y - x) / c0                                         # :570
        if th_store_mask[i]:
            th_out[:, :, k_th] = th_next
            k_th += 1
        if I_store_mask[i]:
            I_out[:, :, k_I] = y + Is
            k_I += 1
        if not Vs_zero:
            theta_s = theta_s + Vs * dt                                # :579-580
        hist = [th_next] + hist[:-1]
        if on_step is not None:
            on_step(i)
    return th_out, I_out


def backward_derivative(x, index, s1, dt):
    """Stencil derivative along the stored-step axis (time_evolution.py:411-420)."""
    w = len(s1)
    out = s1[0] * x[:, :, index]
    for k in range(1, w - 1):
        out = out + s1[k] * x[:, :, index - k]
    return out / dt


def time_evolution(problem, noise=None, core=evolve):
    """Restatement of time_evolution (time_evolution.py:422-458).

    Returns (theta, current, voltage), each (Nj, W, Nt_stored) or None when not stored.
    """
    Nt = problem._Nt()
    store = np.asarray(problem.store_time_steps, bool)
    need_th = problem.store_theta or problem.store_voltage
    need_I = problem.store_current or problem.store_voltage
    th_mask = store.copy() if need_th else np.zeros(Nt, bool)
    I_mask = store.copy() if need_I else np.zeros(Nt, bool)
    Vth_mask, VI_mask = th_mask.copy(), I_mask.copy()
    offset = problem.stencil_width - 1
    c = problem.get_circuit()
    t_ids = np.flatnonzero(store)
    if problem.store_voltage and len(t_ids) > 0:
        ids = (t_ids[:, None] - np.arange(offset)).ravel()
        ids = ids[(ids >= 0) & (ids < Nt)]
        Vth_mask[ids] = True
        if c._has_inductance():
            VI_mask[ids] = True
    th_out, I_out = core(problem, Vth_mask, VI_mask, noise=noise) if noise is not None else \
        core(problem, Vth_mask, VI_mask)
    V = None
    if problem.store_voltage:
        ts = np.flatnonzero(store[Vth_mask])
        s1 = problem.stencil[0]
        V = backward_derivative(th_out, ts + offset, s1, problem._dt())
        if c._has_inductance():
            VI = backward_derivative(I_out, ts + offset, s1, problem._dt())
            Nj = c._Nj()
            V = V + (c.get_inductance() @ VI.reshape((Nj, -1))).reshape(V.shape)
        th_out = np.delete(th_out, np.flatnonzero((Vth_mask & ~th_mask)[Vth_mask]) + offset, axis=2)
        I_out = np.delete(I_out, np.flatnonzero((VI_mask & ~I_mask)[VI_mask]) + offset, axis=2)
    th_out, I_out = th_out[:, :, offset:], I_out[:, :, offset:]
    return (th_out if problem.store_theta else None,
            I_out if problem.store_current else None, V)


def vortex_configuration(A, theta):
    """n = -A round(theta / 2 pi), per stored step (time_evolution.py:734-755)."""
    Nf = A.shape[0]
    Nj, W, S = theta.shape
    r = np.round(theta / (2.0 * np.pi)).reshape(Nj, W * S)
    return (-(A @ r)).reshape(Nf, W, S).astype(int)


def anneal(problem_cls, circuit, time_step=0.5, interval_steps=10, external_flux=0.0, current_sources=0,
           problem_count=1, interval_count=1000, vortex_mobility=0.001, start_T=1.0, T_factor=1.03):
    """Restatement of AnnealingProblem.compute (time_evolution.py:1070-1191) up to, not including,
    its final static (Newton) refinement, with the noise of ``evolve`` (np.random, per call).

    ``problem_cls``: a TimeEvolutionProblem class with the reference's constructor and attributes
    (the reference's own or a mirror of it). Follows the reference literally: each interval
    restarts from config_at_minus_1 = config_at_minus_2 = the last phase; the vortex mobility is
    sum |diff n| / (Nf dt (interval_count - 1)) (:1131-1136); the temperature of a problem is
    divided by T_factor when its mobility exceeds the target v ((N - i) / N)^1.5, else multiplied
    (:1138-1143); then five runs at T = 0 with half the time step (:1171-1178).
    Returns (theta (Nj, W), vortex configuration (Nf, W) at the last step, temperature profiles
    (interval_count, W), vortex mobility (interval_count, W)).
    """
    Nj, Nf = circuit._Nj(), circuit._Nf()
    W = problem_count
    T = start_T * np.ones((1, W, 1))
    f = np.atleast_1d(external_flux)[:, None, None]
    th = np.zeros((Nj, W))
    prob = problem_cls(circuit, time_step_count=interval_steps, time_step=time_step, external_flux=f,
                       current_sources=current_sources, temperature=T, store_current=False, store_voltage=False,
                       stencil_width=3)
    A = circuit.get_cycle_matrix()
    profiles = np.zeros((interval_count, W))
    mobility = np.zeros((interval_count, W))
    for i in range(interval_count):
        prob.temperature = T * np.ones((1, 1, interval_steps))
        prob.config_at_minus_1 = th
        prob.config_at_minus_2 = th.copy()
        theta, _, _ = time_evolution(prob)
        n = vortex_configuration(A, theta)
        mob = np.sum(np.sum(np.abs(np.diff(n, axis=2)), axis=2), axis=0) / (Nf * time_step * (interval_count - 1))
        v = vortex_mobility
        upper = v[i] if np.array(v).size == interval_count else v * ((interval_count - i) / interval_count) ** 1.5
        factor = (mob > upper) * (1 / T_factor) + (mob <= upper) * T_factor
        T = T * factor[..., None]
        th = theta[..., -1]
        profiles[i] = T[0, :, 0]
        mobility[i] = mob
    prob.temperature = np.zeros((1, 1, interval_steps))
    prob.time_step /= 2
    for _ in range(5):
        prob.config_at_minus_1 = th
        prob.config_at_minus_2 = th.copy()
        theta, _, _ = time_evolution(prob)
        th = theta[..., -1]
    return th, vortex_configuration(A, theta)[:, :, -1], profiles, mobility
