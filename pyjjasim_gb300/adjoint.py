"""Gradients of time-evolution losses by a checkpointed adjoint on the GPU.

No counterpart in the reference (pyjjasim has no derivatives). For a loss that is linear in
the phases at chosen steps, L_w = sum_n <G_n[:, w], theta_n[:, w]> (time-averaged voltages are
of this form), ``AdjointRun`` returns dL/dIc (per junction and problem), dL/dIs and dL/df.

Forward: the usual GPU time stepping, keeping the phase history (theta_{s-1}, theta_{s-2}) at
the start of every segment of ~sqrt(Nt) steps. Backward: segments in reverse; each is
recomputed from its checkpoint with every phase kept on the device, then walked backwards with
``jja_adjoint_step`` (one face-space solve per step with the same factor, K being symmetric).
Memory: 2 sqrt(Nt) + sqrt(Nt) phase arrays instead of Nt. Cost: forward + recompute + adjoint,
about three forward passes. Stencil width 3 (the reference default) only.
"""
import ctypes
import math

import numpy as np

from . import _native as N
from .backend import GpuSimulation, _torch
from .problem import TimeEvolutionProblem

__all__ = ["AdjointRun", "time_averaged_voltage_weights", "vortex_flow_weights", "TimeAveragedVoltageLoss"]


def time_averaged_voltage_weights(problem, t1, t2, junctions=None):
    """Loss weights of the mean voltage over ``junctions`` between steps t1 < t2:
    V = (theta_t2 - theta_t1) / (dt (t2 - t1)) averaged over the junctions (per problem)."""
    Nj, W = problem.get_circuit()._Nj(), problem.get_problem_count()
    mask = np.ones(Nj, bool) if junctions is None else np.zeros(Nj, bool)
    if junctions is not None:
        mask[junctions] = True
    w = np.zeros((Nj, W))
    w[mask] = 1.0 / (mask.sum() * problem._dt() * (t2 - t1))
    return {t2: w, t1: -w}


def vortex_flow_weights(problem, t1, t2, junctions, signs=None):
    """Loss weights of the mean vortex flow across a line of junctions between steps t1 < t2.

    A vortex crossing a junction advances its phase by 2 pi (the Josephson relation, V =
    d theta / dt in the reference's units), so the net number of vortices crossing the line
    per unit time is sum_j s_j (theta_j(t2) - theta_j(t1)) / (2 pi dt (t2 - t1)), with s_j = +-1
    orienting each junction across the line (``signs``, default +1). The time-averaged vortex
    flow is linear in the phases, as the adjoint requires; its discrete counterpart is the
    change of the vortex configurations (TimeEvolutionResult.get_vortex_configuration)."""
    Nj, W = problem.get_circuit()._Nj(), problem.get_problem_count()
    junctions = np.asarray(junctions)
    s = np.ones(len(junctions)) if signs is None else np.asarray(signs, np.float64)
    w = np.zeros((Nj, W))
    np.add.at(w, junctions, (s / (2 * np.pi * problem._dt() * (t2 - t1)))[:, None])
    return {t2: w, t1: -w}


class AdjointRun:
    """Forward pass with checkpoints (``loss`` per problem); ``backward()`` gives the gradients."""

    def __init__(self, problem, loss_weights, checkpoint_every=None, Ic=None, noise="philox", seed=None,
                 **factor_options):
        if problem.stencil_width != 3:
            raise NotImplementedError("the adjoint supports stencil width 3 (the reference default) only")
        self.torch = torch = _torch()
        self.sim = sim = GpuSimulation(problem, noise=noise, seed=seed, Ic=Ic, **factor_options)
        if sim.theta_s is not None:
            raise NotImplementedError("the adjoint does not support voltage sources")
        self.problem = problem
        self.Nj, self.Nf, self.W = sim.Nj, sim.Nf, sim.W
        Nt = problem._Nt()
        S = checkpoint_every or max(1, int(math.ceil(math.sqrt(Nt))))
        self.segments = [(s0, min(Nt, s0 + S)) for s0 in range(0, Nt, S)]
        self.Nt = Nt
        dev = sim.dev
        self.G = {int(n): torch.from_numpy(np.array(np.broadcast_to(g, (self.Nj, self.W)), np.float64,
                                                    order="C")).to(dev)
                  for n, g in loss_weights.items()}
        for n in self.G:
            if not 0 <= n < Nt:
                raise ValueError(f"loss step {n} outside [0, {Nt})")
        self._forward()

    def _forward(self):
        torch, sim = self.torch, self.sim
        # every tensor operation runs on the simulation's stream, ordered with its kernels
        with torch.cuda.device(sim.dev), torch.cuda.stream(sim.stream):
            loss = torch.zeros(self.W, dtype=torch.float64, device=sim.dev)
            self.checkpoints = []
            for s0, s1 in self.segments:
                self.checkpoints.append([h.clone() for h in sim.history()])
                steps = [n for n in sorted(self.G) if s0 <= n < s1]
                slots = np.full(s1 - s0, -1, np.int64)
                for k, n in enumerate(steps):
                    slots[n - s0] = k
                th = torch.empty((len(steps), self.Nj, self.W), dtype=torch.float64, device=sim.dev) if steps else None
                sim.run(s1 - s0, slots, None, th, None, use_graph=True)
                for k, n in enumerate(steps):
                    loss += (self.G[n] * th[k]).sum(0)
        sim.synchronize()
        self.loss = loss

    def backward(self):
        """dL_w/dIc (Nj, W), dL_w/dIs (Nj, W), dL_w/df (Nf, W) as device tensors."""
        torch, sim = self.torch, self.sim
        with torch.cuda.device(sim.dev), torch.cuda.stream(sim.stream):
            return self._backward(torch, sim)

    def _backward(self, torch, sim):
        lib = N.lib()
        z = lambda: torch.zeros((self.Nj, self.W), dtype=torch.float64, device=sim.dev)
        mu, cs = [z() for _ in range(3)], [z() for _ in range(3)]
        usum, musum, gIc = z(), z(), z()
        h = ctypes.c_void_p(sim.stream.cuda_stream)
        # one segment buffer for all segments: the same addresses every time, so the captured
        # graphs of the recomputation and of the adjoint walk are replayed, not recaptured
        S = max(s1 - s0 for s0, s1 in self.segments)
        seg_all = torch.empty((S + 2, self.Nj, self.W), dtype=torch.float64, device=sim.dev)
        for (s0, s1), ck in reversed(list(zip(self.segments, self.checkpoints))):
            L = s1 - s0
            sim.set_history(ck, s0)
            seg = seg_all[:L + 2]
            seg[0].copy_(ck[1])
            seg[1].copy_(ck[0])
            sim.run(L, None, None, seg[2:], None, use_graph=True, store_all=True)
            # the segment's adjoint steps, last to first, in one library call
            a = N.AdjointSegmentArgs()
            a.seg, a.s0, a.L, a.Nt = seg.data_ptr(), s0, L, self.Nt
            gtab = (ctypes.c_void_p * L)(*[self.G[n].data_ptr() if n in self.G else None for n in range(s0, s1)])
            a.G = ctypes.cast(gtab, ctypes.POINTER(ctypes.c_void_p))
            for k in range(3):
                a.mu[k], a.cos[k] = mu[k].data_ptr(), cs[k].data_ptr()
            a.usum, a.musum, a.gIc = usum.data_ptr(), musum.data_ptr(), gIc.data_ptr()
            a.use_graph = 1
            N.check(lib.jja_adjoint_segment(sim.plan.handle, ctypes.byref(a), h))
        gf = torch.empty((self.Nf, self.W), dtype=torch.float64, device=sim.dev)
        N.check(lib.jja_adjoint_flux(sim.plan.handle, ctypes.c_void_p(usum.data_ptr()),
                                     ctypes.c_void_p(gf.data_ptr()), h))
        sim.synchronize()
        return {"Ic": gIc, "Is": -musum, "f": gf}


def _problem_from(setup, f, bias):
    c = setup["circuit"]
    base = np.asarray(setup["base"], np.float64)
    Is = base[:, None, None] * np.asarray(bias, np.float64)[None, :, None]
    return TimeEvolutionProblem(c, time_step=setup["dt"], time_step_count=setup["Nt"], current_sources=Is,
                                external_flux=np.asarray(f, np.float64)[:, :, None], store_time_steps=[setup["Nt"] - 1],
                                store_voltage=False, store_current=False)


def _make_loss_function():
    torch = _torch()

    class _Loss(torch.autograd.Function):
        """Time-averaged array voltage of W problems as a differentiable function of their
        critical currents Ic (Nj, W), frustrations f (Nf, W) and bias amplitudes (W,).

        ``setup``: dict(circuit=..., dt=..., Nt=..., base=(Nj,) source pattern (the bias
        multiplies it), t1=..., t2=..., junctions=index array or None)."""

        @staticmethod
        def forward(ctx, Ic, f, bias, setup):
            prob = _problem_from(setup, f.detach().cpu().numpy(), bias.detach().cpu().numpy())
            weights = time_averaged_voltage_weights(prob, setup["t1"], setup["t2"], setup.get("junctions"))
            run = AdjointRun(prob, weights, Ic=Ic.detach().cpu().numpy(), noise="philox",
                             seed=setup.get("seed", 0))
            ctx.run, ctx.base = run, torch.as_tensor(np.asarray(setup["base"], np.float64))
            return run.loss.to(Ic.device)

        @staticmethod
        def backward(ctx, grad):
            g = ctx.run.backward()
            gr = grad.to(g["Ic"].device)[None, :]
            gIs = g["Is"] * gr
            gbias = (ctx.base.to(gIs.device)[:, None] * gIs).sum(0)
            dev = grad.device
            return (g["Ic"] * gr).to(dev), (g["f"] * gr).to(dev), gbias.to(dev), None

    return _Loss


class _LazyLoss:
    """``TimeAveragedVoltageLoss.apply(Ic, f, bias, setup)`` (torch imported on first use)."""

    _fn = None

    def apply(self, *args):
        if _LazyLoss._fn is None:
            _LazyLoss._fn = _make_loss_function()
        return _LazyLoss._fn.apply(*args)


TimeAveragedVoltageLoss = _LazyLoss()
