"""Adjoint gradients against central finite differences of the CPU oracle.

Loss: time-averaged voltage over the horizontal junctions between two steps, per problem.
Parameters: per-problem critical currents Ic (Nj, W), frustration f (Nf, W), bias (W,).
Directional derivatives <grad, d> for random d are compared with (L(p + h d) - L(p - h d)) / 2h
computed by the oracle (the reference's algorithm, pinned to its golden outputs), run per
problem with that problem's Ic.
"""
import numpy as np
import pytest

from oracle import rcsj_oracle
from pyjjasim_gb300 import SquareArray, TimeEvolutionProblem
from pyjjasim_gb300.adjoint import AdjointRun, TimeAveragedVoltageLoss, time_averaged_voltage_weights

pytestmark = pytest.mark.gpu
NX, NT, T1, T2, W = 5, 240, 119, 239, 2


def _setup():
    rng = np.random.default_rng(21)
    c = SquareArray(NX, NX)
    Nj, Nf = c.junction_count(), c.face_count()
    Ic = rng.lognormal(0.0, 0.2, (Nj, W))
    f = rng.uniform(0.05, 0.2, (Nf, W))
    bias = np.array([1.25, 1.6])
    base = c.current_base(0.0)
    horiz = np.arange(NX * (NX - 1))
    return c, Ic, f, bias, base, horiz


def _problem(c, f, bias, base):
    Is = base[:, None, None] * bias[None, :, None]
    return TimeEvolutionProblem(c, time_step=0.05, time_step_count=NT, current_sources=Is,
                                external_flux=f[:, :, None], store_time_steps=[T1, T2], store_voltage=False,
                                store_current=False)


def _oracle_loss(c, Ic, f, bias, base, horiz):
    out = []
    for w in range(W):
        cw = SquareArray(NX, NX)
        cw.set_critical_current(Ic[:, w])
        p = _problem(cw, f[:, [w]], bias[[w]], base)
        th, _, _ = rcsj_oracle.time_evolution(p)
        out.append((th[horiz, 0, 1] - th[horiz, 0, 0]).mean() / (0.05 * (T2 - T1)))
    return np.array(out)


def test_adjoint_matches_oracle_finite_differences():
    c, Ic, f, bias, base, horiz = _setup()
    prob = _problem(c, f, bias, base)
    run = AdjointRun(prob, time_averaged_voltage_weights(prob, T1, T2, horiz), Ic=Ic)
    L0 = _oracle_loss(c, Ic, f, bias, base, horiz)
    np.testing.assert_allclose(run.loss.cpu().numpy(), L0, rtol=1e-9, atol=1e-12)
    g = {k: v.cpu().numpy() for k, v in run.backward().items()}
    rng = np.random.default_rng(4)
    h = 1e-4
    dIc, df, db = rng.standard_normal(Ic.shape), rng.standard_normal(f.shape), rng.standard_normal(W)
    cases = [("Ic", (Ic + h * dIc, f, bias), (Ic - h * dIc, f, bias), (g["Ic"] * dIc).sum(0)),
             ("f", (Ic, f + h * df, bias), (Ic, f - h * df, bias), (g["f"] * df).sum(0)),
             ("bias", (Ic, f, bias + h * db), (Ic, f, bias - h * db), (g["Is"] * base[:, None]).sum(0) * db)]
    for name, plus, minus, ad in cases:
        fd = (_oracle_loss(c, *plus, base, horiz) - _oracle_loss(c, *minus, base, horiz)) / (2 * h)
        scale = np.abs(fd).max() + 1e-12
        assert np.abs(ad - fd).max() <= 1e-5 * scale + 1e-9, f"{name}: adjoint {ad} vs finite differences {fd}"


def test_autograd_wrapper_matches_adjoint_run():
    import torch
    c, Ic, f, bias, base, horiz = _setup()
    setup = dict(circuit=c, dt=0.05, Nt=NT, base=base, t1=T1, t2=T2, junctions=horiz)
    tIc = torch.tensor(Ic, requires_grad=True)
    tf = torch.tensor(f, requires_grad=True)
    tb = torch.tensor(bias, requires_grad=True)
    loss = TimeAveragedVoltageLoss.apply(tIc, tf, tb, setup)
    (loss * torch.tensor([1.0, 2.0], dtype=torch.float64)).sum().backward()
    prob = _problem(c, f, bias, base)
    run = AdjointRun(prob, time_averaged_voltage_weights(prob, T1, T2, horiz), Ic=Ic)
    g = {k: v.cpu().numpy() for k, v in run.backward().items()}
    wts = np.array([1.0, 2.0])
    np.testing.assert_allclose(tIc.grad.numpy(), g["Ic"] * wts, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(tf.grad.numpy(), g["f"] * wts, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(tb.grad.numpy(), (g["Is"] * base[:, None]).sum(0) * wts, rtol=1e-10, atol=1e-14)


def test_vortex_flow_gradient_matches_finite_differences():
    """Gradient of the mean vortex flow across the middle row of horizontal junctions (a
    linear loss of the phases) against central finite differences of the oracle."""
    from pyjjasim_gb300.adjoint import vortex_flow_weights
    c, Ic, f, bias, base, horiz = _setup()
    # horizontal junctions j = y (NX - 1) + x of the middle row: the line that vortices cross
    # when the horizontal bias drives them across the array
    line = (NX // 2) * (NX - 1) + np.arange(NX - 1)
    prob = _problem(c, f, bias, base)
    run = AdjointRun(prob, vortex_flow_weights(prob, T1, T2, line), Ic=Ic)
    g = {k: v.cpu().numpy() for k, v in run.backward().items()}

    def flow(Icx, fx, bx):
        out = []
        for w in range(W):
            cw = SquareArray(NX, NX)
            cw.set_critical_current(Icx[:, w])
            th, _, _ = rcsj_oracle.time_evolution(_problem(cw, fx[:, [w]], bx[[w]], base))
            out.append((th[line, 0, 1] - th[line, 0, 0]).sum() / (2 * np.pi * 0.05 * (T2 - T1)))
        return np.array(out)

    np.testing.assert_allclose(run.loss.cpu().numpy(), flow(Ic, f, bias), rtol=1e-9, atol=1e-12)
    rng = np.random.default_rng(9)
    h = 1e-4
    dIc, df = rng.standard_normal(Ic.shape), rng.standard_normal(f.shape)
    for name, plus, minus, ad in (("Ic", (Ic + h * dIc, f, bias), (Ic - h * dIc, f, bias), (g["Ic"] * dIc).sum(0)),
                                  ("f", (Ic, f + h * df, bias), (Ic, f - h * df, bias), (g["f"] * df).sum(0))):
        fd = (flow(*plus) - flow(*minus)) / (2 * h)
        scale = np.abs(fd).max() + 1e-12
        assert np.abs(ad - fd).max() <= 1e-5 * scale + 1e-9, f"{name}: adjoint {ad} vs finite differences {fd}"


@pytest.mark.parametrize("W_s,tuning", [(32, {"subtree_rows": 32}), (8, {"subtree_rows": 32})])
def test_adjoint_with_subtree_sweeps_matches_level_sweeps(W_s, tuning):
    """The adjoint's face solves run through the same sweep schedule as the forward steps: with
    the bottom subtrees solved in shared memory (one warp per subtree and 32 problems, or packs
    of subtrees of one shape below 32 problems) the gradients equal those of the level-only
    schedule up to summation order."""
    rng = np.random.default_rng(5)
    c = SquareArray(24, 24)
    Nj, Nf = c.junction_count(), c.face_count()
    Ic = rng.lognormal(0.0, 0.2, (Nj, W_s))
    Is = c.current_base(0.0)[:, None, None] * np.linspace(1.1, 1.5, W_s)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=160, current_sources=Is, external_flux=0.12,
                                store_time_steps=[79, 159], store_voltage=False, store_current=False)
    weights = time_averaged_voltage_weights(prob, 79, 159, np.arange(24 * 23))
    grads = []
    for t in (tuning, {"subtree_rows": -1}):
        run = AdjointRun(prob, weights, Ic=Ic, ordering="nd", tuning=t)
        grads.append({k: v.cpu().numpy() for k, v in run.backward().items()})
    for k in grads[0]:
        a, b = grads[0][k], grads[1][k]
        assert np.abs(a - b).max() <= 1e-9 * max(1.0, np.abs(b).max()), k
