"""GPU parity: the CUDA path against the reference's golden vectors and the CPU oracle.

Tolerances (FP64 on both sides, different summation orders in the face-space solve):
* T = 0 trajectories: |theta_gpu - theta_ref| <= 1e-9 * max(1, |theta_ref|), the bar the
  reference comparison is held to over a 2000-step run;
* noisy runs with the reference's own noise draws replayed (noise="numpy"): same bar;
* the face-space solve alone: relative 1e-11 against scipy's sparse direct solve.
"""
import numpy as np
import pytest
import scipy.sparse.linalg

import golden_cases as gc
from oracle import rcsj_oracle
from pyjjasim_gb300 import TimeEvolutionProblem, backend
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray

pytestmark = pytest.mark.gpu
TRAJ_RTOL = 1e-9


def close(actual, desired, rtol=TRAJ_RTOL):
    scale = max(1.0, float(np.abs(desired).max()))
    err = float(np.abs(actual - desired).max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:.1e} * {scale:.3e}"


@pytest.mark.parametrize("name", gc.case_names())
def test_golden_parity(name):
    z = gc.load(name)
    prob = gc.problem(z)
    s = gc.seed(z)
    if s is not None:
        np.random.seed(s)
    res = prob.compute(noise="numpy")
    close(res.get_theta(), z["theta"])
    close(res.get_current(), z["current"])
    close(res.get_voltage(), z["voltage"], rtol=1e-8)
    assert np.array_equal(res.get_vortex_configuration(), z["vortex"])
    # derived observables of the GPU result (node solves amplify the phase error a little)
    for obs in ("phase", "josephson_energy", "supercurrent", "cycle_current", "flux", "magnetic_energy", "potential",
                "capacitive_energy", "energy"):
        close(getattr(res, "get_" + obs)(), z["obs_" + obs], rtol=1e-6)


@pytest.mark.parametrize("make,W", [(lambda: SquareArray(9, 13), 1), (lambda: SquareArray(20, 20), 37),
                                    (lambda: HoneycombArray(6, 5), 64), (lambda: TriangularArray(7, 6), 3),
                                    (lambda: SquareArray(64, 64), 40)])
def test_face_solve_matches_scipy(make, W):
    c = make()
    c.set_inductance(0.05)
    dt = 0.05
    A, K = P.face_matrix(c, dt)
    b = np.random.default_rng(W).standard_normal((K.shape[0], W))
    x = backend.solve_faces(c, dt, b)
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b).reshape(x.shape)
    close(x, ref, rtol=1e-11)


@pytest.mark.parametrize("make", [lambda: SquareArray(60, 47), lambda: HoneycombArray(25, 21),
                                  lambda: TriangularArray(33, 40)])
@pytest.mark.parametrize("ordering", ["nd", "mmd"])
@pytest.mark.parametrize("pack_rows", [0, 8, 48])
def test_face_solve_w1_packs(make, ordering, pack_rows):
    """W = 1 packs of small supernodes (one per lane, interleaved values) on every level where
    they fit (pack_min_warps 1): the solve against scipy, and against the same plan without packs."""
    c = make()
    c.set_inductance(0.05)
    A, K = P.face_matrix(c, 0.05)
    b = np.random.default_rng(pack_rows).standard_normal(K.shape[0])
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    x = backend.solve_faces(c, 0.05, b, ordering=ordering, tuning={"pack_rows": pack_rows, "pack_min_warps": 1})
    x0 = backend.solve_faces(c, 0.05, b, ordering=ordering, tuning={"pack_rows": -1})
    close(x, ref, rtol=1e-11)
    close(x, x0, rtol=1e-12)


@pytest.mark.parametrize("make", [lambda: SquareArray(40, 33), lambda: HoneycombArray(12, 9),
                                  lambda: TriangularArray(15, 14)])
def test_node_space_solve_on_device(make):
    """Node phases of a GPU result: the node-space solve M_r M_r^T x = M_r y on the GPU against
    SuperLU on the host (the reference's Circuit.Msq_solve), last node grounded."""
    from pyjjasim_gb300 import observables
    c = make()
    y = np.random.default_rng(4).standard_normal((c.junction_count(), 7))
    b = c.get_cut_matrix() @ y
    close(observables.msq_solve(c, b), c.Msq_solve(b), rtol=1e-11)
    close(observables.msq_solve(c, b[:, 0]), c.Msq_solve(b[:, 0]), rtol=1e-11)


def _mixed_problem(c, W, Nt, seed):
    rng = np.random.default_rng(seed)
    Nj, Nf = c.junction_count(), c.face_count()
    Is = c.current_base(0.3)[:, None, None] * np.linspace(0.2, 1.4, W)[None, :, None]
    f = rng.uniform(0, 0.5, (Nf, 1, 1))
    th1 = rng.standard_normal((Nj, W)) * 0.3
    return TimeEvolutionProblem(c, time_step=0.07, time_step_count=Nt, current_sources=Is, external_flux=f,
                                config_at_minus_1=th1, config_at_minus_2=th1 * 0.98,
                                store_time_steps=np.arange(0, Nt, 7))


@pytest.mark.parametrize("make,W", [(lambda: HoneycombArray(5, 6), 5), (lambda: TriangularArray(6, 5), 7),
                                    (lambda: SquareArray(11, 17), 33)])
def test_against_oracle(make, W):
    c = make()
    c.set_capacitance(0.3)
    c.set_inductance(0.2)
    prob = _mixed_problem(c, W, 300, W)
    th_o, I_o, V_o = rcsj_oracle.time_evolution(prob)
    res = prob.compute()
    close(res.get_theta(), th_o)
    close(res.get_current(), I_o)
    close(res.get_voltage(), V_o, rtol=1e-8)


def test_w1_packs_against_oracle():
    """One problem (W = 1) with packs on every level where they fit, against the oracle."""
    c = SquareArray(31, 26)
    c.set_capacitance(0.3)
    c.set_inductance(0.2)
    prob = _mixed_problem(c, 1, 300, 11)
    th_o, I_o, V_o = rcsj_oracle.time_evolution(prob)
    res = prob.compute(tuning={"pack_min_warps": 1}, ordering="mmd")
    close(res.get_theta(), th_o)
    close(res.get_current(), I_o)
    close(res.get_voltage(), V_o, rtol=1e-8)


def test_device_sine_accuracy():
    """The junction kernels' sine (64-bit fixed point + FP32, no FP64 instruction): equal, bit
    for bit, to the same source run on the host (whose error the CPU tests bound over many more
    points), within 1.2e-16 absolute of numpy's sine for |x| < 2^62, near zeros of sine within
    1e-18 absolute plus 2 ulps, NaN from 2^62 on."""
    import torch
    from pyjjasim_gb300 import _native as N
    c = SquareArray(3, 3)
    pl = P.get_plan(c, 0.05, 1, 3, ((1.0, -1.0, 0.0), (1.0, -2.0, 1.0)))
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 200000), rng.uniform(-4, 4, 100000),
                        np.arange(-3000, 3000) * (np.pi / 2048) + rng.uniform(-1e-9, 1e-9, 6000),
                        np.array([0.0, -0.0, 1e-300, np.pi, -np.pi, 2 * np.pi, 1e5, 3e5, -7e6, 1e15, 2.0 ** 62]),
                        rng.uniform(-2e5, 2e5, 10000), 10.0 ** rng.uniform(-12, 18, 50000)])
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    pl.eval_sin(xd.data_ptr(), out.data_ptr(), x.size)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    host = np.empty_like(x)
    N.check(N.lib().jja_sin_host(N.ptr(x), N.ptr(host), None, x.size))
    assert np.array_equal(got, host, equal_nan=True)
    fin = np.abs(x) < 2.0 ** 62
    assert np.all(np.isnan(got[~fin]))
    ref = np.sin(x[fin])
    err = np.abs(got[fin] - ref)
    i = int(np.argmax(err))
    assert err.max() <= 1.2e-16, f"max abs error {err.max():.3e} at x={x[fin][i]!r}: {got[fin][i]!r} vs {ref[i]!r}"
    xf = x[fin]
    near = (np.abs(xf - np.round(xf / np.pi) * np.pi) < np.pi / 4096) & (np.abs(xf) < 2e5)
    assert near.sum() > 100 and np.all(err[near] <= 1e-18 + 2.3e-16 * np.abs(ref[near]))


def test_graph_and_eager_paths_agree():
    c = SquareArray(24, 24)
    W = 16
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0, 2, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=400, current_sources=Is, external_flux=0.25,
                                store_time_steps=[399])
    th_g, _ = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, use_graph=True)
    th_e, _ = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, use_graph=False)
    close(th_g, th_e, rtol=1e-11)


@pytest.mark.parametrize("groups", [2, 3])
def test_problem_groups_match_one_chain(groups):
    """The step run as independent groups of problems on their own streams (forked from and
    joined back into the call's stream, inside and outside captured graphs) gives the one-chain
    trajectory: thermal noise keyed by (junction-problem, step), time-dependent sources, stored
    steps and the adjoint-style store_all path all see the same global problem index."""
    c = SquareArray(21, 19)
    c.set_inductance(0.1)
    W, Nt = 96, 120
    Is = lambda i: c.current_base(0.0)[:, None] * (np.linspace(0.2, 1.6, W)[None, :] + 0.1 * np.sin(0.05 * i))
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, current_sources=Is, external_flux=0.2,
                                temperature=0.01, store_time_steps=np.arange(0, Nt, 9))
    th1, I1 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, seed=5,
                                          tuning={"groups": 1})
    th2, I2 = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, seed=5,
                                          tuning={"groups": groups})
    close(th2, th1, rtol=1e-10)
    close(I2, I1, rtol=1e-10)


@pytest.mark.parametrize("W,groups", [(5, 0), (70, 3)])
def test_store_all_matches_per_step_slots(W, groups):
    """Storing every step with slots derived on the device (graph replays) gives the same
    phases and currents as per-step slots from the host (eager launches), also with the step
    split into groups of problems."""
    import torch
    c = SquareArray(17, 13)
    L = 150
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.5, 1.5, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=L, current_sources=Is, external_flux=0.2)
    out = []
    for store_all in (False, True):
        sim = backend.GpuSimulation(prob, tuning={"groups": groups})
        th = torch.empty((L, c.junction_count(), W), dtype=torch.float64, device=sim.dev)
        I = torch.empty_like(th)
        with torch.cuda.stream(sim.stream):
            if store_all:
                sim.run(L, None, None, th, I, use_graph=True, store_all=True)
            else:
                sim.run(L, np.arange(L), np.arange(L), th, I, use_graph=False)
        sim.synchronize()
        out.append((th.cpu().numpy(), I.cpu().numpy()))
    close(out[1][0], out[0][0], rtol=1e-12)
    close(out[1][1], out[0][1], rtol=1e-12)


def test_full_size_kirchhoff_invariants():
    """IV-sweep shape at full size (128x128 array, W=512): A theta + 2 pi f = 0 (no inductance)
    and current conservation M (I - Is) = 0 after many steps; both are size-independent."""
    c = SquareArray(128, 128)
    W, Nt, f = 512, 200, 0.25
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0, 2, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, current_sources=Is, external_flux=f,
                                store_time_steps=[Nt - 1], store_voltage=False)
    res = prob.compute()
    th = res.get_theta()[:, :, 0]
    I = res.get_current()[:, :, 0]
    A, M = c.get_cycle_matrix(), c.get_cut_matrix()
    kvl = A @ th + 2 * np.pi * f
    assert np.abs(kvl).max() < 1e-9 * max(1.0, np.abs(th).max())
    kcl = M @ (I - Is[:, :, 0])
    assert np.abs(kcl).max() < 1e-9
    assert np.all(np.isfinite(th))


def test_philox_noise_statistics():
    """On-device noise: mean-square junction voltage at T>0, C=0, Is=0 follows the
    fluctuation amplitude; checked against the oracle driven by its own normal draws."""
    c = SquareArray(16, 16)
    W, Nt, T = 64, 400, 0.05
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, temperature=T * np.ones((1, W, 1)),
                                store_time_steps=np.arange(Nt // 2, Nt), store_current=False)
    res = prob.compute(noise="philox", seed=1234)
    V = res.get_voltage()
    rng = np.random.default_rng(0)
    th_o, _, V_o = rcsj_oracle.time_evolution(prob, noise=lambda i: rng.standard_normal((c.junction_count(), W)))
    ms_gpu, ms_cpu = float(np.mean(V ** 2)), float(np.mean(V_o ** 2))
    assert abs(ms_gpu - ms_cpu) < 0.03 * ms_cpu
    # different seeds give different paths, the same seed the same path
    res2 = prob.compute(noise="philox", seed=1234)
    close(res2.get_theta(), res.get_theta(), rtol=1e-10)
