"""Generate tests/golden/adjoint_fd_64x64.npz: finite differences of the oracle on the
adjoint workload, the reference values the GPU adjoint is checked against.

Workload (the benchmark's adjoint configuration): SquareArray(64, 64), per-junction critical
currents Ic ~ lognormal(0, 0.2) (the first two problems of the benchmark's draw,
np.random.default_rng(2024).lognormal(0, 0.2, (Nj, 64))), f = 0.1 on every face, DC bias
1.2 x current_base(0), T = 0, dt = 0.05. Loss per problem and horizon T (5000, the workload's,
and 400): the mean voltage of the horizontal junctions over steps T/2-1..T-1,
(theta_{T-1} - theta_{T/2-1}) / (dt T/2) averaged over those junctions (the reference's IV-curve
quantity, examples/time_evolution_example_2_IV_curve.py). Both horizons come from the same runs
(the first 400 steps of a 5000-step trajectory are the 400-step trajectory).

For random directions dIc (Nj per problem), df (Nf per problem) and dbias = 1, the central
differences (L(p + h d) - L(p - h d)) / 2h at h = 1e-3 ... 1e-7 are computed with the CPU
oracle (oracle/rcsj_oracle.py, pinned to the reference's own outputs), one problem per run, in
parallel worker processes. The fixture stores the inputs, the directions, the losses and every
difference; tests/test_adjoint_long.py compares the GPU adjoint's directional derivatives with
them. In this running state the loss is smooth only very close to the parameters: at 5000 steps
the differences settle only for h <= 1e-6, at 400 steps for every h.

Usage:  python tests/golden/make_adjoint_fd.py   (about a minute on 8 cores)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N, DT, F0, BIAS = 64, 0.05, 0.1, 1.2
HORIZONS = (5000, 400)
NT = max(HORIZONS)
HS = (1e-3, 1e-4, 1e-5, 1e-6, 1e-7)
OUT = os.path.join(HERE, "adjoint_fd_64x64.npz")


def loss(Ic, f, bias):
    """Oracle losses of one problem at every horizon: Ic (Nj,), f (Nf,), bias scalar."""
    import pyjjasim_gb300 as G
    from oracle import rcsj_oracle
    c = G.SquareArray(N, N)
    c.set_critical_current(np.asarray(Ic, np.float64))
    Is = c.current_base(0.0)[:, None, None] * float(bias)
    store = sorted({T // 2 - 1 for T in HORIZONS} | {T - 1 for T in HORIZONS})
    p = G.TimeEvolutionProblem(c, time_step=DT, time_step_count=NT, current_sources=Is,
                               external_flux=np.asarray(f, np.float64)[:, None, None], store_time_steps=store,
                               store_voltage=False, store_current=False)
    th, _, _ = rcsj_oracle.time_evolution(p)
    horiz = np.arange(N * (N - 1))
    return [float((th[horiz, 0, store.index(T - 1)] - th[horiz, 0, store.index(T // 2 - 1)]).mean()
                  / (DT * (T - T // 2))) for T in HORIZONS]


def main():
    import pyjjasim_gb300 as G
    from oracle import parity_jobs as PJ
    c = G.SquareArray(N, N)
    Nj, Nf = c.junction_count(), c.face_count()
    Ic = np.random.default_rng(2024).lognormal(0.0, 0.2, (Nj, 64))[:, :2]
    W = Ic.shape[1]
    rng = np.random.default_rng(5)
    dIc, df = rng.standard_normal((Nj, W)), rng.standard_normal((Nf, W))
    f = np.full((Nf, W), F0)
    jobs = {}
    pool = PJ.pool(min(12, os.cpu_count() or 1))
    for w in range(W):
        jobs[("L0", w)] = pool.apply_async(loss, (Ic[:, w], f[:, w], BIAS))
        for k, h in enumerate(HS):
            for sgn in (1, -1):
                jobs[("Ic", w, k, sgn)] = pool.apply_async(loss, (Ic[:, w] + sgn * h * dIc[:, w], f[:, w], BIAS))
                jobs[("f", w, k, sgn)] = pool.apply_async(loss, (Ic[:, w], f[:, w] + sgn * h * df[:, w], BIAS))
                jobs[("bias", w, k, sgn)] = pool.apply_async(loss, (Ic[:, w], f[:, w], BIAS + sgn * h))
    res = {k: v.get() for k, v in jobs.items()}
    pool.close()
    pool.join()
    res = {k: np.array(v) for k, v in res.items()}
    out = dict(Ic=Ic, dIc=dIc, df=df, f0=F0, bias=BIAS, horizons=np.array(HORIZONS), dt=DT, hs=np.array(HS),
               L0=np.array([res[("L0", w)] for w in range(W)]).T)                      # (horizon, problem)
    for name in ("Ic", "f", "bias"):
        # (horizon, h, problem)
        out["fd_" + name] = np.array([[(res[(name, w, k, 1)] - res[(name, w, k, -1)]) / (2 * h) for w in range(W)]
                                      for k, h in enumerate(HS)]).transpose(2, 0, 1)
    np.savez_compressed(OUT, **out)
    for name in ("Ic", "f", "bias"):
        for i, T in enumerate(HORIZONS):
            print(name, T, out["fd_" + name][i].tolist())
    print("L0", out["L0"].tolist())


if __name__ == "__main__":
    main()
