"""Generate the golden fixtures under tests/golden/ by running the reference pyjjasim.

This script is the only committed code that imports the reference package. It runs
where the reference sources are present (read-only; their directory is given by --ref);
the fixtures it writes (`*.npz`) are what the tests read on machines without it.

Import recipe: the reference imports itself as ``pyjjasim.*`` (pyjjasim/__init__.py),
imports matplotlib at module load (embedded_graph.py:3-4, circuit_visualize.py:3-11),
and calls ``np.asscalar`` (time_evolution.py:322), which numpy removed. So the script
puts a symlink ``pyjjasim -> <ref>`` in a temporary directory on sys.path,
stubs the matplotlib modules and re-adds ``np.asscalar``. Nothing in the reference is
modified; bytecode writing is disabled so its read-only tree is never touched.

Each fixture holds the exact inputs (cycle matrix A, component vectors, source arrays or
the parameters of a source callable, seeds, store masks) and the reference outputs
(theta, current, voltage at the stored steps, the vortex configuration, and the result's
derived observables: node phases and potentials, cycle currents, flux, supercurrent and the
energies), so a test can rebuild the same problem with no reference present.

Usage:  python tests/golden/make_golden.py --ref <reference source directory>
"""
import argparse
import os
import sys
import tempfile
import types
import warnings

import numpy as np
import scipy.sparse

HERE = os.path.dirname(os.path.abspath(__file__))


MATPLOTLIB_STUBS = ["matplotlib", "matplotlib.pyplot", "matplotlib.collections", "matplotlib.animation",
                    "matplotlib.colors", "matplotlib.cm", "matplotlib.patches", "matplotlib.lines",
                    "matplotlib.legend_handler", "matplotlib.text"]


def _stub_attr(name):
    # module metadata (__file__, __path__, ...) stays absent, so tools that walk sys.modules
    # (inspect) see an ordinary module; every other name is a no-op callable
    if name.startswith("__"):
        raise AttributeError(name)
    return lambda *a, **k: None


def import_reference(ref_dir):
    for m in MATPLOTLIB_STUBS:
        mod = types.ModuleType(m)
        mod.__getattr__ = _stub_attr
        sys.modules[m] = mod
    if not hasattr(np, "asscalar"):
        np.asscalar = lambda a: a.item()
    sys.dont_write_bytecode = True
    tmp = tempfile.mkdtemp(prefix="pyjjasim_ref_")
    os.symlink(ref_dir, os.path.join(tmp, "pyjjasim"))
    sys.path.insert(0, tmp)
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    import pyjjasim  # noqa: F401
    return pyjjasim


def csr_parts(prefix, M):
    M = scipy.sparse.csr_matrix(M)
    M.sort_indices()
    return {prefix + "_data": M.data.astype(np.float64), prefix + "_indices": M.indices.astype(np.int64),
            prefix + "_indptr": M.indptr.astype(np.int64), prefix + "_shape": np.array(M.shape, np.int64)}


def circuit_parts(c):
    d = {}
    d.update(csr_parts("A", c.get_cycle_matrix()))
    d.update(csr_parts("M", c.get_cut_matrix()))
    d.update(csr_parts("L", c.get_inductance()))
    x, y = c.get_node_coordinates()
    n1, n2 = c.get_junction_nodes()
    d.update(Ic=c.get_critical_current().copy(), R=c.get_resistance().copy(),
             C=c.get_capacitance().copy(), node_x=np.asarray(x, np.float64), node_y=np.asarray(y, np.float64),
             node1=np.asarray(n1, np.int64), node2=np.asarray(n2, np.int64),
             face_centroid_x=np.asarray(c.get_face_centroids()[0], np.float64),
             face_centroid_y=np.asarray(c.get_face_centroids()[1], np.float64))
    return d


def run_case(pj, name, circuit, dt, Nt, *, f=0.0, Is=0.0, Vs=0.0, T=0.0, seed=None, store=None,
             stencil_width=3, th_m1=None, th_m2=None, th_m3=None, th_m4=None, Is_spec=None, extra=None):
    """Run the reference compute() and save inputs + outputs."""
    kw = dict(time_step=dt, time_step_count=Nt, external_flux=f, current_sources=Is, voltage_sources=Vs,
              temperature=T, store_time_steps=store, stencil_width=stencil_width,
              config_at_minus_1=th_m1, config_at_minus_2=th_m2, config_at_minus_3=th_m3,
              config_at_minus_4=th_m4)
    prob = pj.TimeEvolutionProblem(circuit, **kw)
    if seed is not None:
        np.random.seed(seed)
    res = prob.compute()
    W = prob.get_problem_count()
    d = circuit_parts(circuit)
    d.update(dt=np.float64(dt), Nt=np.int64(Nt), W=np.int64(W), stencil_width=np.int64(stencil_width),
             seed=np.int64(-1 if seed is None else seed), store_mask=prob.get_store_time_steps().copy(),
             theta=res.get_theta(), current=res.current.copy(), voltage=res.get_voltage(),
             vortex=res.get_vortex_configuration())
    # the result's derived observables (time_evolution.py:692-985) at every stored step
    for obs in ("phase", "josephson_energy", "supercurrent", "cycle_current", "flux", "magnetic_energy", "potential",
                "capacitive_energy", "energy"):
        d["obs_" + obs] = np.asarray(getattr(res, "get_" + obs)(), dtype=np.float64)
    # inputs: arrays stored compact (before broadcasting); callables by their parameters
    for key, val in (("f", f), ("Is", Is), ("Vs", Vs), ("T", T)):
        if callable(val):
            continue
        d["in_" + key] = np.array(val, dtype=np.float64)
    for key, val in (("th_m1", th_m1), ("th_m2", th_m2), ("th_m3", th_m3), ("th_m4", th_m4)):
        if val is not None:
            d["in_" + key] = np.array(val, dtype=np.float64)
    if Is_spec is not None:
        for k, v in Is_spec.items():
            d["Is_spec_" + k] = np.asarray(v)
    if extra:
        d.update(extra)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **d)
    print(f"{name}: Nj={circuit.junction_count()} Nf={circuit.face_count()} W={W} Nt={Nt} -> "
          f"{os.path.getsize(path) / 1024:.0f} KB")


def anneal_case(pj, name, circuit, seed, **params):
    """Run the reference AnnealingProblem.compute() and save its inputs, the temperature profiles
    and the vortex configurations it hands to its final static refinement (recorded by wrapping
    TimeEvolutionProblem.get_static_problem at run time; the reference's files are untouched)."""
    handed = []
    orig = pj.TimeEvolutionProblem.get_static_problem

    def record(self, vortex_configuration, *a, **k):
        handed.append(np.array(vortex_configuration, dtype=np.int64))
        return orig(self, vortex_configuration, *a, **k)

    pj.TimeEvolutionProblem.get_static_problem = record
    try:
        np.random.seed(seed)
        status, configs, profiles = pj.AnnealingProblem(circuit, **params).compute()
    finally:
        pj.TimeEvolutionProblem.get_static_problem = orig
    d = circuit_parts(circuit)
    d.update(seed=np.int64(seed), temperature_profiles=profiles, status=np.asarray(status),
             final_vortex=np.stack(handed, axis=1),
             static_theta=np.stack([cfg.get_theta() for cfg in configs], axis=1))
    for k, v in params.items():
        d["param_" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: Nj={circuit.junction_count()} W={params.get('problem_count', 1)} "
          f"intervals={params.get('interval_count')}")


def every(Nt, k):
    m = np.zeros(Nt, bool)
    m[::k] = True
    m[-1] = True
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="directory of the reference pyjjasim sources")
    ap.add_argument("--anneal-only", action="store_true", help="write only the AnnealingProblem fixtures")
    ap.add_argument("--static-only", action="store_true",
                    help="write only the StaticProblem and AnnealingProblem fixtures")
    args = ap.parse_args()
    pj = import_reference(args.ref)
    if args.anneal_only:
        return anneal_fixtures(pj)
    if args.static_only:
        static_fixtures(pj)
        return anneal_fixtures(pj)

    # Lattice fixtures: cycle matrices, cut matrices and current_base for the three lattice kinds.
    lat = {}
    for kind, cls, sizes in (("square", pj.SquareArray, [(2, 2), (3, 3), (4, 7), (10, 10), (7, 4)]),
                             ("honeycomb", pj.HoneycombArray, [(1, 1), (2, 2), (3, 4), (4, 3)]),
                             ("triangular", pj.TriangularArray, [(2, 2), (3, 3), (4, 5), (5, 4)])):
        for (nx, ny) in sizes:
            c = cls(nx, ny)
            key = f"{kind}_{nx}x{ny}"
            for k, v in circuit_parts(c).items():
                lat[key + "__" + k] = v
            lat[key + "__cb0"] = c.current_base(0.0)
            lat[key + "__cb90"] = c.current_base(np.pi / 2)
            lat[key + "__cb30"] = c.current_base(np.pi / 6)
    np.savez_compressed(os.path.join(HERE, "lattices.npz"), **lat)
    print("lattices.npz written")

    # Config 1 exactly: SquareArray(10,10), f=0.1, Is=0.5*current_base(0), T=0, dt=0.05, 2000 steps.
    a = pj.SquareArray(10, 10)
    Is = 0.5 * a.current_base(0.0)
    run_case(pj, "c1_square10_dc", a, 0.05, 2000, f=0.1, Is=Is[:, None, None], store=every(2000, 25))

    # Config 2 shape, reduced: C=1, L=0.1, AC bias callable, T=0.01, seeded noise (Nj <= 500: fresh draws).
    a = pj.SquareArray(8, 8)
    a.set_capacitance(1.0)
    a.set_inductance(0.1)
    base = a.current_base(0.0)
    dt = 0.05
    Is_fn = lambda i: (base * (0.8 + 0.3 * np.sin(2 * np.pi * 0.05 * i * dt)))[:, None]
    run_case(pj, "c2_square8_cl_ac_noise", a, dt, 400, f=0.1, Is=Is_fn, T=0.01, seed=0,
             store=every(400, 10), Is_spec=dict(base=base, dc=0.8, ac=0.3, freq=0.05))

    # Config 3 shape, reduced: W=8 IV sweep, f=0.25, bias linspace(0, 2, 8), T=0.
    a = pj.SquareArray(12, 12)
    Is = a.current_base(0.0)[:, None, None] * np.linspace(0, 2, 8)[None, :, None]
    run_case(pj, "c3_square12_iv_w8", a, 0.05, 600, f=0.25, Is=Is, store=every(600, 50))

    # Nj > 500: the reference reuses the previous draw with permuted rows on steps i % 3 != 0.
    a = pj.SquareArray(17, 17)
    Is = 0.5 * a.current_base(0.0)
    run_case(pj, "c4_square17_noise_perm", a, 0.05, 30, f=0.1, Is=Is[:, None, None] * np.array([1.0, 0.6])[None, :, None],
             T=0.02, seed=3, store=every(30, 4))

    # Config 4 shape, reduced: lognormal Ic, bias 1.2, W=4 (Ic is per circuit, W shares it).
    rng = np.random.default_rng(7)
    a = pj.SquareArray(8, 8)
    a.set_critical_current(rng.lognormal(0.0, 0.2, a.junction_count()))
    Is = 1.2 * a.current_base(0.0)
    run_case(pj, "c5_square8_lognormal_ic", a, 0.05, 500, f=np.array([0.1, 0.15, 0.2, 0.3])[None, :, None],
             Is=Is[:, None, None], store=every(500, 25))

    # Honeycomb and triangular lattices.
    a = pj.HoneycombArray(4, 3)
    Is = 0.7 * a.current_base(0.0)
    run_case(pj, "c6_honeycomb4x3", a, 0.05, 300, f=0.2, Is=Is[:, None, None] * np.array([1.0, 1.5])[None, :, None],
             store=every(300, 10))
    a = pj.TriangularArray(5, 4)
    Is = 0.6 * a.current_base(0.0)
    run_case(pj, "c7_triangular5x4", a, 0.05, 300, f=0.15, Is=Is[:, None, None], store=every(300, 10))

    # Stencil widths 4 and 5, with capacitance and voltage sources (theta_s path).
    for sw in (4, 5):
        a = pj.SquareArray(6, 6)
        a.set_capacitance(0.5)
        Nj = a.junction_count()
        rng = np.random.default_rng(sw)
        Vs = 0.01 * rng.standard_normal(Nj)
        Is = 0.4 * a.current_base(0.0)
        th0 = 0.1 * rng.standard_normal(Nj)
        run_case(pj, f"c8_square6_stencil{sw}_vs", a, 0.05, 200, f=0.1, Is=Is[:, None, None], Vs=Vs[:, None, None],
                 store=every(200, 10), stencil_width=sw, th_m1=th0)

    # Mutual inductance matrix and junction current sources not derived from node currents.
    a = pj.SquareArray(6, 6)
    Nj = a.junction_count()
    rng = np.random.default_rng(11)
    Lm = scipy.sparse.diags(np.full(Nj, 0.3)) + scipy.sparse.diags(np.full(Nj - 1, 0.05), 1) + \
        scipy.sparse.diags(np.full(Nj - 1, 0.05), -1)
    a.set_inductance(Lm.tocsc())
    Is = 0.3 * rng.standard_normal(Nj)
    run_case(pj, "c9_square6_mutual_l", a, 0.05, 200, f=0.05, Is=Is[:, None, None], store=every(200, 5))

    # Time-dependent arrays for f and T (full (N, W, Nt) arrays), noise with time-dependent T, W=3.
    a = pj.SquareArray(7, 5)
    Nt = 120
    Nf, Nj = a.face_count(), a.junction_count()
    fa = 0.1 + 0.05 * np.sin(np.arange(Nt) * 0.1)[None, None, :] * np.ones((Nf, 3, 1))
    Ta = np.linspace(0.0, 0.02, Nt)[None, None, :] * np.ones((1, 3, 1))
    Is = 0.5 * a.current_base(0.0)
    th1 = 0.2 * np.random.default_rng(5).standard_normal((Nj, 3))
    th2 = th1 - 0.01
    run_case(pj, "c10_square7x5_timedep", a, 0.1, Nt, f=fa, Is=Is[:, None, None], T=Ta, seed=9,
             store=every(Nt, 3), th_m1=th1, th_m2=th2)
    anneal_fixtures(pj)


def static_case(pj, name, circuit, Is, f, n, initial_guess=None, **kw):
    """Run the reference's StaticProblem(...).compute() (the Newton iteration static_compute,
    static_problem.py:1400-1515, started from approximate() unless a guess is given) and save its
    inputs, the initial guess, the solution, the status and the iteration record."""
    prob = pj.StaticProblem(circuit, current_sources=Is, external_flux=f, vortex_configuration=n)
    theta0 = prob.approximate().get_theta() if initial_guess is None else np.asarray(initial_guess, np.float64)
    config, status, info = prob.compute(initial_guess=initial_guess, **kw)
    d = circuit_parts(circuit)
    d.update(in_Is=np.broadcast_to(np.asarray(Is, np.float64), (circuit.junction_count(),)).copy(),
             in_f=np.broadcast_to(np.asarray(f, np.float64), (circuit.face_count(),)).copy(),
             in_n=np.broadcast_to(np.asarray(n, np.int64), (circuit.face_count(),)).copy(),
             theta0=np.asarray(theta0, np.float64), guess_given=np.int64(initial_guess is not None),
             theta=config.get_theta().copy(), current=config.get_current().copy(),
             vortex=config.get_vortex_configuration().astype(np.int64), status=np.int64(status),
             iterations=np.int64(info.get_number_of_iterations()), residuals=info.get_residual().copy(),
             is_target=info.get_is_target_vortex_configuration().astype(np.int64))
    for k, v in kw.items():
        d["param_" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: Nj={circuit.junction_count()} status={status} iterations={info.get_number_of_iterations()}")


def static_fixtures(pj):
    # Newton iteration of static problems (StaticProblem.compute, static_problem.py:559-607):
    # converging cases (s1-s3, s6) and two the reference's iteration gives up on (s4: bias above
    # the critical current, no static state; s5: a poor initial guess)
    a = pj.SquareArray(8, 7)
    n = np.zeros(a.face_count(), int)
    n[a.face_count() // 2] = 1
    static_case(pj, "s1_square8x7_vortex", a, 0.3 * a.current_base(0.0), 0.05, n)
    h = pj.HoneycombArray(4, 4)
    h.set_inductance(0.3)
    static_case(pj, "s2_honeycomb4x4_inductance", h, 0.0, 0.2, 0)
    t = pj.TriangularArray(5, 5)
    t.set_critical_current(np.random.default_rng(8).lognormal(0.0, 0.2, t.junction_count()))
    static_case(pj, "s3_triangular5x5_disorder", t, 0.3 * t.current_base(np.pi / 2), 0.05, 0)
    a = pj.SquareArray(6, 6)
    static_case(pj, "s4_square6_overbias", a, 3.0 * a.current_base(0.0), 0.0, 0)
    a = pj.SquareArray(7, 6)
    a.set_inductance(np.random.default_rng(9).uniform(0.05, 0.4, a.junction_count()))
    rng = np.random.default_rng(10)
    guess = rng.uniform(-0.3, 0.3, a.junction_count())
    static_case(pj, "s5_square7x6_guess", a, 0.2 * a.current_base(0.3), rng.uniform(0, 0.3, a.face_count()), 0,
                initial_guess=guess, tol=1e-12, maxiter=40)
    a = pj.SquareArray(12, 10)
    a.set_inductance(0.2)
    n = np.zeros(a.face_count(), int)
    n[40] = 1
    static_case(pj, "s6_square12x10_inductance_vortex", a, 0.2 * a.current_base(0.0), 0.05, n)


def anneal_fixtures(pj):
    # AnnealingProblem (time_evolution.py:1070-1191): per-problem temperatures driven by the
    # measured vortex mobility (they diverge between problems with these parameters)
    anneal_case(pj, "a1_square6x5_anneal", pj.SquareArray(6, 5), 5, time_step=0.5, interval_steps=8,
                interval_count=40, problem_count=3, external_flux=0.25, vortex_mobility=0.05, start_T=1.0,
                T_factor=1.1)


if __name__ == "__main__":
    main()
