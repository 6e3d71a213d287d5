"""TimeEvolutionProblem / TimeEvolutionResult with the reference's interface.

Mirrors pyjjasim time_evolution.py so that code written against the reference runs
unchanged here, with the per-step core executed on the GPU:

* ``TimeEvolutionProblem`` (time_evolution.py:20-409): same constructor arguments,
  problem-count inference (:110-116), broadcasting of sources to (N, W, Nt) views or
  kept callables (:119-130), store masks (:132-140, 384-399), stencils (:401-408),
  initial conditions (:144-149, 327-332) and per-step accessors ``_f/_Is/_Vs/_T``
  (:342-356).
* ``time_evolution`` (time_evolution.py:422-458): widens the store masks so the
  voltage stencil has its previous steps, calls the core, derives V, strips helper
  steps. The core is the GPU backend (``pyjjasim_gb300.backend.time_evolution_core``).
* ``TimeEvolutionResult`` (time_evolution.py:597-1067): theta / current / voltage /
  vortex configuration accessors and the derived observables (node phases and potentials,
  cycle currents, flux, supercurrent, energies; :692-985) with the same shapes and errors.
  For results of the GPU core the node-space solves of the phases and potentials run on the
  GPU (``pyjjasim_gb300.observables``).
"""
import numpy as np

__all__ = ["DefaultCPR", "TimeEvolutionProblem", "TimeEvolutionResult", "time_evolution",
           "ThetaNotStored", "CurrentNotStored", "VoltageNotStored", "DataAtTimepointNotStored"]


class DefaultCPR:
    """Current-phase relation Ic*sin(theta) (static_problem.py:77-85)."""

    def eval(self, Ic, theta):
        return Ic * np.sin(theta)

    def d_eval(self, Ic, theta):
        return Ic * np.cos(theta)

    def i_eval(self, Ic, theta):
        return Ic * (1.0 - np.cos(theta))


def stencil(width):
    """Backward stencils (first derivative, second derivative) of width 3, 4 or 5."""
    if width == 3:
        return (1.0, -1.0, 0.0), (1.0, -2.0, 1.0)
    if width == 4:
        return (1.5, -2.0, 0.5, 0.0), (2.0, -5.0, 4.0, -1.0)
    if width == 5:
        return (11.0 / 6, -3.0, 1.5, -1.0 / 3, 0.0), (35.0 / 12, -26.0 / 3, 9.5, -14.0 / 3, 11.0 / 12)
    raise ValueError(f"stencil width must be 3, 4 or 5 (equals {width})")


class TimeEvolutionProblem:
    """W time-evolution problems on one Josephson circuit (see time_evolution.py:20-92).

    Arrays are broadcast to (Nf|Nj, W, Nt) read-only views; callables f(i) -> (N, W)
    are evaluated per step. ``compute()`` runs the GPU backend.
    """

    def __init__(self, circuit, time_step=0.05, time_step_count=1000, current_phase_relation=None,
                 external_flux=0.0, current_sources=0.0, voltage_sources=0.0, temperature=0.0,
                 store_time_steps=None, store_theta=True, store_voltage=True, store_current=True,
                 config_at_minus_1=None, config_at_minus_2=None, config_at_minus_3=None,
                 config_at_minus_4=None, stencil_width=3):
        self.circuit = circuit
        self.time_step = time_step
        self.time_step_count = time_step_count
        self.current_phase_relation = DefaultCPR() if current_phase_relation is None else current_phase_relation

        def count(x):
            s = np.shape(x(0) if callable(x) else x)
            return s[1] if len(s) > 1 else 1

        self.problem_count = max(count(external_flux), count(current_sources), count(voltage_sources),
                                 count(temperature))
        Nj, Nf, W, Nt = circuit._Nj(), circuit._Nf(), self.problem_count, time_step_count

        def prep(x, N):
            return x if callable(x) else np.broadcast_to(np.array(x), (N, W, Nt))

        self._f_is_timedep = self._is_timedep(external_flux)
        self.external_flux = prep(external_flux, Nf)
        self._Is_is_timedep = self._is_timedep(current_sources)
        self.current_sources = prep(current_sources, Nj)
        self._Vs_is_timedep = self._is_timedep(voltage_sources)
        self.voltage_sources = prep(voltage_sources, Nj)
        self._T_is_timedep = self._is_timedep(temperature)
        self.temperature = prep(temperature, Nj)

        self.store_time_steps = np.ones(Nt, dtype=bool)
        self.store_time_steps = self._to_time_point_mask(store_time_steps)
        self.store_theta, self.store_voltage, self.store_current = store_theta, store_voltage, store_current
        if not (store_theta or store_voltage or store_current):
            raise ValueError("No output is stored")
        if np.sum(self.store_time_steps) == 0:
            raise ValueError("No output is stored")
        self.stencil_width = stencil_width
        self.stencil = stencil(stencil_width)
        zeros = np.zeros((Nj, W), dtype=np.double)
        self.config_at_minus_1 = self._get_config(config_at_minus_1, zeros, (Nj, W))
        self.config_at_minus_2 = self._get_config(config_at_minus_2, self.config_at_minus_1, (Nj, W))
        if stencil_width >= 4:
            self.config_at_minus_3 = self._get_config(config_at_minus_3, self.config_at_minus_2, (Nj, W))
        if stencil_width >= 5:
            self.config_at_minus_4 = self._get_config(config_at_minus_4, self.config_at_minus_3, (Nj, W))

    # --- public getters (time_evolution.py:172-301) -----------------------------------------
    def get_problem_count(self):
        return self.problem_count

    def get_circuit(self):
        return self.circuit

    def get_time_step(self):
        return self.time_step

    def get_time_step_count(self):
        return self.time_step_count

    def get_current_phase_relation(self):
        return self.current_phase_relation

    def get_static_problem(self, vortex_configuration, problem_nr=0, time_step=0):
        """A StaticProblem with this problem's sources and flux of one problem at one step
        (time_evolution.py:151-172); it computes on the GPU."""
        from .static import StaticProblem
        return StaticProblem(self.circuit, current_sources=self._Is(time_step)[:, problem_nr].copy(),
                             external_flux=self._f(time_step)[:, problem_nr].copy(),
                             vortex_configuration=vortex_configuration,
                             current_phase_relation=self.current_phase_relation)

    def get_external_flux(self):
        return self.external_flux

    def get_current_sources(self):
        return self.current_sources

    def get_voltage_sources(self):
        return self.voltage_sources

    def get_temperature(self):
        return self.temperature

    def get_store_time_steps(self):
        return self.store_time_steps

    def get_store_theta(self):
        return self.store_theta

    def get_store_voltage(self):
        return self.store_voltage

    def get_store_current(self):
        return self.store_current

    def get_time(self):
        return np.arange(self._Nt(), dtype=np.double) * self._dt()

    def compute(self, backend="gb300", **options):
        """Run the time evolution and return a TimeEvolutionResult.

        ``backend="gb300"`` (the only backend) executes the per-step core on the GPU.
        ``options`` are forwarded to it (``noise="philox"|"numpy"``, ``seed``,
        ``precision``, ``device``).
        """
        if backend != "gb300":
            raise ValueError(f"unknown backend {backend!r}; this package provides 'gb300' only")
        return time_evolution(self, **options)

    # --- internal accessors (time_evolution.py:315-408) -------------------------------------
    def _Nt(self):
        return self.time_step_count

    def _Nt_s(self):
        return int(np.sum(self.store_time_steps))

    def _dt(self):
        return self.time_step

    @staticmethod
    def _get_config(cur, prev, shape):
        cur = prev.copy() if cur is None else cur
        if hasattr(cur, "get_theta"):
            cur = cur.get_theta()
        return np.asarray(cur, dtype=np.double).reshape(shape)

    @staticmethod
    def _is_timedep(x):
        if callable(x):
            return True
        s = np.shape(x)
        return len(s) > 0 and s[-1] > 1

    def _step_value(self, x, N, i):
        if callable(x):
            return np.broadcast_to(x(i), (N, self.problem_count))
        return x[:, :, i]

    def _f(self, i):
        return self._step_value(self.external_flux, self.circuit._Nf(), i)

    def _Is(self, i):
        return self._step_value(self.current_sources, self.circuit._Nj(), i)

    def _Vs(self, i):
        return self._step_value(self.voltage_sources, self.circuit._Nj(), i)

    def _T(self, i):
        return self._step_value(self.temperature, self.circuit._Nj(), i)

    def _cp(self, theta):
        return self.current_phase_relation.eval(self.circuit._Ic()[:, None], theta)

    def _icp(self, theta):
        return self.current_phase_relation.i_eval(self.circuit._Ic()[:, None], theta)

    def _to_time_point_mask(self, time_points):
        if time_points is None:
            time_points = self.store_time_steps
        time_points = np.array(time_points)
        if time_points.dtype != bool:
            try:
                m = np.zeros(self._Nt(), dtype=bool)
                m[time_points] = True
                time_points = m
            except Exception:
                raise ValueError("Invalid store_time_steps; must be None, mask, slice or index array")
        return time_points


def _stencil_derivative(x_tm, index, s1, dt):
    """Backward-stencil derivative at stored slots ``index`` of a time-major (slots, Nj, W)
    array, returned time-major (time_evolution.py:411-420, same operation order)."""
    out = x_tm[index]          # a copy (integer-array index)
    if s1[0] != 1.0:           # 1 x is exact: skip the pass
        out *= s1[0]
    for k in range(1, len(s1) - 1):
        for j, i in enumerate(index):   # slot by slot: no temporary of all slots
            if s1[k] == -1.0:           # -1 x then add: the same rounding as a subtraction
                np.subtract(out[j], x_tm[i - k], out=out[j])
            else:
                out[j] += s1[k] * x_tm[i - k]
    out /= dt
    return out


def _select_slots(x, slots):
    """x[:, :, slots] for a (Nj, W, S) array, kept as a view of its time-major storage when
    the slots form a contiguous range."""
    tm = x.transpose(2, 0, 1)
    if len(slots) and np.all(np.diff(slots) == 1):
        return tm[slots[0]:slots[-1] + 1].transpose(1, 2, 0)
    return tm[slots].transpose(1, 2, 0)


def time_evolution(problem, core=None, **options):
    """Driver around the GPU core: masks, core call, voltage (time_evolution.py:422-458).

    ``core`` replaces the GPU core with another function of the same signature (tests use
    this to check the masks and post-processing on a machine without a GPU)."""
    on_device = core is None
    if core is None:
        from .backend import time_evolution_core as core
    Nt = problem._Nt()
    store = np.asarray(problem.store_time_steps, bool)
    th_mask = store.copy() if (problem.store_theta or problem.store_voltage) else np.zeros(Nt, bool)
    I_mask = store.copy() if (problem.store_current or problem.store_voltage) else np.zeros(Nt, bool)
    Vth_mask, VI_mask = th_mask.copy(), I_mask.copy()
    t_ids = np.flatnonzero(store)
    c = problem.get_circuit()
    offset = problem.stencil_width - 1
    if problem.store_voltage and len(t_ids) > 0:
        ids = (t_ids[:, None] - np.arange(offset)).ravel()
        ids = ids[(ids >= 0) & (ids < Nt)]
        Vth_mask[ids] = True
        if c._has_inductance():
            VI_mask[ids] = True
    th_out, I_out = core(problem, Vth_mask, VI_mask, **options)
    V = None
    if problem.store_voltage:
        ts = np.flatnonzero(store[Vth_mask])
        s1, dt = problem.stencil[0], problem._dt()
        V = _stencil_derivative(th_out.transpose(2, 0, 1), ts + offset, s1, dt)
        if c._has_inductance():
            VI = _stencil_derivative(I_out.transpose(2, 0, 1), ts + offset, s1, dt)
            Nj = c._Nj()
            VI = np.ascontiguousarray(VI.transpose(1, 2, 0)).reshape((Nj, -1))
            V = V + (c.get_inductance() @ VI).reshape((Nj, -1, len(ts))).transpose(2, 0, 1)
        V = V.transpose(1, 2, 0)
    # keep the slots of steps stored for their own sake (the reference deletes the helper
    # slots and the initial conditions, time_evolution.py:451-455)
    th_keep = offset + np.flatnonzero(th_mask[Vth_mask])
    I_keep = offset + np.flatnonzero(I_mask[VI_mask])
    th_out = _select_slots(th_out, th_keep) if problem.store_theta else None
    I_out = _select_slots(I_out, I_keep) if problem.store_current else None
    res = TimeEvolutionResult(problem, th_out, I_out, V)
    res.node_solves_on_device = on_device
    return res


class ThetaNotStored(Exception):
    pass


class CurrentNotStored(Exception):
    pass


class VoltageNotStored(Exception):
    pass


class DataAtTimepointNotStored(Exception):
    pass


class TimeEvolutionResult:
    """Stored theta / current / voltage of a time evolution (time_evolution.py:597-1067)."""

    def __init__(self, problem, theta, current, voltage):
        self.problem = problem
        Nj, W, Nt_s = problem.circuit._Nj(), problem.get_problem_count(), problem._Nt_s()
        for name, arr, flag in (("theta", theta, problem.store_theta), ("current", current, problem.store_current),
                                ("voltage", voltage, problem.store_voltage)):
            if flag and arr.shape != (Nj, W, Nt_s):
                raise ValueError(f"{name} must have shape {(Nj, W, Nt_s)}; has shape {arr.shape}")
        self.theta = theta if problem.store_theta else None
        self.current = current if problem.store_current else None
        self.voltage = voltage if problem.store_voltage else None
        s = problem.store_time_steps.astype(int)
        self.time_point_indices = np.cumsum(s) - s
        # node phases / potentials solve M_r M_r^T x = b: with the GPU core's results on the GPU
        # (pyjjasim_gb300.observables), else with SuperLU on the host as the reference does
        self.node_solves_on_device = False

    def _msq_solve(self, b):
        c = self.get_circuit()
        if self.node_solves_on_device:
            from .observables import msq_solve
            return msq_solve(c, b)
        return c.Msq_solve(b)

    def get_problem_count(self):
        return self.problem.get_problem_count()

    def get_circuit(self):
        return self.problem.get_circuit()

    def _time_point_index(self, time_points):
        if time_points is None:
            time_points = self.problem.store_time_steps
        if not np.all(self.problem.store_time_steps[time_points]):
            raise DataAtTimepointNotStored("Queried a timepoint that is not stored during time evolution simulation.")
        return self.time_point_indices[time_points]

    def _th(self, tp):
        if self.theta is None:
            raise ThetaNotStored("Cannot query theta; quantity is not stored during time evolution simulation.")
        return self.theta[:, :, self._time_point_index(tp)]

    def _V(self, tp):
        if self.voltage is None:
            raise VoltageNotStored("Cannot query voltage; quantity is not stored during time evolution simulation.")
        return self.voltage[:, :, self._time_point_index(tp)]

    def _I(self, tp):
        if self.current is None:
            raise CurrentNotStored("Cannot query current; quantity is not stored during time evolution simulation.")
        return self.current[:, :, self._time_point_index(tp)]

    def _select(self, select_time_points, N, func, is_zero=False):
        # filled time-major (contiguous copies) and returned as the (N, W, T) view
        sel = np.flatnonzero(self.problem._to_time_point_mask(select_time_points))
        if is_zero:
            return np.zeros((N, self.get_problem_count(), len(sel)), dtype=np.double)
        out = np.empty((len(sel), N, self.get_problem_count()), dtype=np.double)
        for k, tp in enumerate(sel):
            out[k] = func(tp)
        return out.transpose(1, 2, 0)

    def get_theta(self, select_time_points=None):
        return self._select(select_time_points, self.get_circuit()._Nj(), self._th)

    def get_current(self, select_time_points=None):
        return self._select(select_time_points, self.get_circuit()._Nj(), self._I)

    def get_voltage(self, select_time_points=None):
        return self._select(select_time_points, self.get_circuit()._Nj(), self._V)

    # observables derived from the stored quantities (time_evolution.py:692-985), same formulas
    def get_phase(self, select_time_points=None):
        """Node phases (Nn, W, T), last node grounded: solves M M^T phi = M theta (:692-714)."""
        c = self.get_circuit()
        M, Nj = c.get_cut_matrix(), c._Nj()
        func = lambda tp: self._msq_solve(M @ self._th(tp).reshape(Nj, -1))
        try:
            return self._select(select_time_points, c._Nn(), func)
        except ThetaNotStored:
            raise ThetaNotStored("Cannot compute phi; requires theta to be stored in TimeEvolutionConfig")

    def get_josephson_energy(self, select_time_points=None):
        """Ic (1 - cos theta) per junction (:757-777)."""
        func = lambda tp: self.problem._icp(self._th(tp))
        try:
            return self._select(select_time_points, self.get_circuit()._Nj(), func)
        except ThetaNotStored:
            raise ThetaNotStored("Cannot compute Josephson energy EJ; requires theta to be stored in TimeEvolutionConfig")

    def get_supercurrent(self, select_time_points=None):
        """Ic sin theta per junction (:797-817)."""
        func = lambda tp: self.problem._cp(self._th(tp))
        try:
            return self._select(select_time_points, self.get_circuit()._Nj(), func)
        except ThetaNotStored:
            raise ThetaNotStored("Cannot compute supercurrent Isup; requires theta to be stored in TimeEvolutionConfig")

    def get_cycle_current(self, select_time_points=None):
        """Cycle currents J with I = A^T J + Is: solves A A^T J = A (I - Is) (:819-841)."""
        c = self.get_circuit()
        A = c.get_cycle_matrix()
        func = lambda tp: c.Asq_solve(A @ (self._I(tp) - self.problem._Is(tp)))
        try:
            return self._select(select_time_points, c._Nf(), func)
        except CurrentNotStored:
            raise CurrentNotStored("Cannot compute cycle-current J; requires current to be stored in TimeEvolutionConfig")

    def get_flux(self, select_time_points=None):
        """Flux through faces, f + A L I / (2 pi) (:843-866)."""
        c = self.get_circuit()
        A = c.get_cycle_matrix()
        func = lambda tp: self.problem._f(tp) + A @ (c._L() @ self._I(tp)) / (2 * np.pi)
        try:
            return self._select(select_time_points, c._Nf(), func)
        except CurrentNotStored:
            raise CurrentNotStored("Cannot compute magnetic flux; requires current to be stored in TimeEvolutionConfig")

    def get_magnetic_energy(self, select_time_points=None):
        """L I^2 / 2 per junction (:868-890)."""
        c = self.get_circuit()
        func = lambda tp: 0.5 * c._L() @ (self._I(tp) ** 2)
        try:
            return self._select(select_time_points, c._Nj(), func, is_zero=not c._has_inductance())
        except CurrentNotStored:
            raise CurrentNotStored("Cannot compute magnetic energy EM; requires current to be stored in TimeEvolutionConfig")

    def get_potential(self, select_time_points=None):
        """Node potentials (Nn, W, T), last node grounded: solves M M^T U = M V (:910-937)."""
        c = self.get_circuit()
        M, Nj = c.get_cut_matrix(), c._Nj()
        func = lambda tp: self._msq_solve(M @ self._V(tp).reshape(Nj, -1))
        try:
            return self._select(select_time_points, c._Nn(), func)
        except VoltageNotStored:
            raise VoltageNotStored("Cannot compute electric potential U; requires voltage to be stored in "
                                   "TimeEvolutionConfig")

    def get_capacitive_energy(self, select_time_points=None):
        """C V^2 / 2 per junction (:939-963)."""
        c = self.get_circuit()
        C = c._C()
        func = lambda tp: 0.5 * C[:, None] * self._V(tp) ** 2
        try:
            return self._select(select_time_points, c._Nj(), func, is_zero=not c._has_capacitance())
        except VoltageNotStored:
            raise VoltageNotStored("Cannot compute capacitive energy EC; requires voltage to be stored in "
                                   "TimeEvolutionConfig")

    def get_energy(self, select_time_points=None):
        """Josephson + magnetic + capacitive energy per junction (:965-985)."""
        return self.get_josephson_energy(select_time_points) + self.get_magnetic_energy(select_time_points) + \
            self.get_capacitive_energy(select_time_points)

    def get_vortex_configuration(self, select_time_points=None):
        A = self.get_circuit().get_cycle_matrix()
        func = lambda tp: -A @ np.round(self._th(tp) / (2.0 * np.pi))
        try:
            return self._select(select_time_points, self.get_circuit()._Nf(), func).astype(int)
        except ThetaNotStored:
            raise ThetaNotStored("Cannot compute n; requires theta to be stored in TimeEvolutionConfig")
