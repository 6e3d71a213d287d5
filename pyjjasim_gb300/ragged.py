"""Ragged batches: problems on different circuits stepped together in one launch sequence.

The reference batches W problems only when they share one circuit (the W axis of
``TimeEvolutionProblem``, time_evolution.py:20-116); different lattices need separate
``compute()`` calls. Here a batch of problems on different circuits (square, honeycomb,
triangular arrays of different sizes, each possibly with several problems) is stepped as ONE
system: the disjoint union of all (problem, w) copies of their circuits. Its cycle matrix and
face-space matrix are block diagonal, so one nested-dissection factorisation yields a forest
whose trees' levels are merged, and every time step is one sequence of level launches over all
problems at once, with the per-problem state laid out back to back (W = 1 in the union).

Large batches are split into a few parts of about equal size, each its own union, factor and
simulation, stepped concurrently on their own streams: each part's launch chain fills the SMs
the other leaves idle at its latency-bound levels (measured on GB300, 32 problems with 4.5M
junctions: one union 1.81 ms per step, two concurrent parts 1.20 ms).

Restrictions: all problems share the time step, step count, stencil width and store mask
(``RaggedBatch`` raises otherwise), and use the default current-phase relation.
"""
import functools
import threading

import numpy as np
import scipy.sparse

from .circuit import Circuit
from .problem import TimeEvolutionProblem, TimeEvolutionResult, time_evolution

__all__ = ["RaggedBatch"]

PART_FROM_JUNCTIONS = 1 << 20    # batches of at least this many junctions (all copies) split in parts ...
PART_JUNCTIONS = 1 << 19         # ... of about this many junctions each, 2 to MAX_PARTS of them
MAX_PARTS = 8
# From this many junctions (all parts) the parts' packed levels take one lane per supernode: the
# concurrent parts give the levels warps enough (measured on GB300, 31M junctions in 8 parts:
# 4.80 ms per step with one lane, 4.99 with the library's per-level choice; 4.5M junctions in 8
# parts: 0.91 against 0.82 ms)
ONE_LANE_FROM_JUNCTIONS = 1 << 24
_SEED_STRIDE = 0x632BE59BD9B4E019   # parts draw thermal noise from distinct Philox streams


def _in_threads(fns):
    """Call every function in its own thread; re-raise the first exception in the caller."""
    errors = []

    def guard(fn):
        try:
            fn()
        except BaseException as e:
            errors.append(e)

    threads = [threading.Thread(target=guard, args=(fn,)) for fn in fns]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]


def _geometry(c):
    x, y = c.get_node_coordinates()
    n1, n2 = c.get_junction_nodes()
    if x is None or n1 is None:
        raise ValueError("ragged batches need circuits with node coordinates and junction nodes")
    return np.asarray(x, float), np.asarray(y, float), np.asarray(n1), np.asarray(n2)


def default_parts(n_junctions):
    """Concurrent parts of a batch with this many junctions (all copies): one union below 2^20
    junctions, else one part per ~2^19 junctions, at least 2 and at most 8 (measured on GB300 with
    4.5M junctions: 2 parts 1.03 ms per step, 4 parts 0.86, 8 parts 0.80; 31M junctions: 8 parts
    5.1 ms, 12 parts 5.2, 16 parts 5.5)."""
    if n_junctions < PART_FROM_JUNCTIONS:
        return 1
    return int(min(MAX_PARTS, max(2, -(-n_junctions // PART_JUNCTIONS))))


class RaggedBatch:
    """A list of TimeEvolutionProblems (any circuits) computed together on the GPU.

    ``parts``: the number of concurrent unions (default: ``default_parts`` of the total junction
    count); problems are assigned whole, largest first, to the part with the fewest junctions."""

    def __init__(self, problems, parts=None):
        if not problems:
            raise ValueError("empty batch")
        p0 = problems[0]
        for p in problems:
            if p._dt() != p0._dt() or p._Nt() != p0._Nt() or p.stencil_width != p0.stencil_width:
                raise ValueError("all problems of a ragged batch need the same time step, step count and stencil")
            if not np.array_equal(np.asarray(p.store_time_steps), np.asarray(p0.store_time_steps)):
                raise ValueError("all problems of a ragged batch need the same store mask")
            if (p.store_theta, p.store_current, p.store_voltage) != (p0.store_theta, p0.store_current,
                                                                     p0.store_voltage):
                raise ValueError("all problems of a ragged batch need the same store flags")
        self.problems = list(problems)
        size = [p.get_circuit()._Nj() * p.get_problem_count() for p in self.problems]
        if parts is None:
            parts = default_parts(sum(size))
        parts = max(1, min(int(parts), len(self.problems)))
        if parts == 1:
            self._build_union()
            self.parts = [self]
            return
        load = [0] * parts
        members = [[] for _ in range(parts)]
        for i in sorted(range(len(self.problems)), key=lambda i: -size[i]):
            k = int(np.argmin(load))
            members[k].append(i)
            load[k] += size[i]
        self.part_members = [sorted(m) for m in members]
        self.parts = [RaggedBatch([self.problems[i] for i in m], parts=1) for m in self.part_members]
        self.Nj = sum(q.Nj for q in self.parts)
        self.Nf = sum(q.Nf for q in self.parts)

    # the union of all (problem, w) copies -------------------------------------------------
    def _build_union(self):
        A_blocks, M_blocks, L_blocks = [], [], []
        Ic, R, C, xs, ys, n1s, n2s = [], [], [], [], [], [], []
        self.slices = []            # per problem: list over w of (junction slice, face slice)
        j0 = f0 = n0 = 0
        x_off = 0.0
        for p in self.problems:
            c = p.get_circuit()
            Nj, Nf, W = c._Nj(), c._Nf(), p.get_problem_count()
            x, y, n1, n2 = _geometry(c)
            width = (x.max() - x.min()) if len(x) else 0.0
            Lmat = scipy.sparse.csr_matrix(c._L())
            per_w = []
            for w in range(W):
                A_blocks.append(scipy.sparse.csr_matrix(c.get_cycle_matrix()))
                M_blocks.append(scipy.sparse.csr_matrix(c.get_cut_matrix()))
                L_blocks.append(Lmat)
                Ic.append(c._Ic())
                R.append(c._R())
                C.append(c._C())
                xs.append(x - x.min() + x_off)
                ys.append(y)
                n1s.append(n1 + n0)
                n2s.append(n2 + n0)
                per_w.append((slice(j0, j0 + Nj), slice(f0, f0 + Nf)))
                j0 += Nj
                f0 += Nf
                n0 += len(x)
                x_off += width + 3.0        # a gap: the union's components never touch
            self.slices.append(per_w)
        self.Nj, self.Nf = j0, f0
        self.circuit = Circuit(scipy.sparse.block_diag(A_blocks, format="csc"), critical_current=np.concatenate(Ic),
                               resistance=np.concatenate(R), capacitance=np.concatenate(C),
                               inductance=scipy.sparse.block_diag(L_blocks, format="csc"),
                               cut_matrix=scipy.sparse.block_diag(M_blocks, format="csc"),
                               node_x=np.concatenate(xs), node_y=np.concatenate(ys), node1=np.concatenate(n1s),
                               node2=np.concatenate(n2s))

    def _union_source(self, getter_name, timedep_name, rows):
        """Concatenate one source over all (problem, w) copies: array (N, 1, 1) or callable."""
        timedep = any(getattr(p, timedep_name) for p in self.problems)

        def at(i):
            parts = []
            for p, per_w in zip(self.problems, self.slices):
                v = np.broadcast_to(getattr(p, getter_name)(i), (rows(p), p.get_problem_count()))
                parts.extend(v[:, w] for w in range(len(per_w)))
            return np.concatenate(parts)

        if timedep:
            return lambda i: at(i)[:, None]
        return at(0)[:, None, None]

    def union_problem(self):
        """The union of all problems as one TimeEvolutionProblem (W = 1): a batch of one part."""
        if len(self.parts) > 1:
            raise ValueError("this batch runs as several parts: use parts[k].union_problem() or simulations()")
        p0 = self.problems[0]
        nj = lambda p: p.get_circuit()._Nj()
        nf = lambda p: p.get_circuit()._Nf()
        hist = {}
        for k in range(1, p0.stencil_width):
            parts = []
            for p, per_w in zip(self.problems, self.slices):
                h = np.broadcast_to(getattr(p, f"config_at_minus_{k}"), (nj(p), p.get_problem_count()))
                parts.extend(h[:, w] for w in range(len(per_w)))
            hist[f"config_at_minus_{k}"] = np.concatenate(parts)[:, None]
        return TimeEvolutionProblem(
            self.circuit, time_step=p0._dt(), time_step_count=p0._Nt(),
            external_flux=self._union_source("_f", "_f_is_timedep", nf),
            current_sources=self._union_source("_Is", "_Is_is_timedep", nj),
            voltage_sources=self._union_source("_Vs", "_Vs_is_timedep", nj),
            temperature=self._union_source("_T", "_T_is_timedep", nj),
            store_time_steps=p0.store_time_steps, store_theta=p0.store_theta, store_voltage=p0.store_voltage,
            store_current=p0.store_current, stencil_width=p0.stencil_width, **hist)

    def _split(self, res):
        """Per-problem results of this union's result."""
        out = []
        for p, per_w in zip(self.problems, self.slices):
            def gather(arr):
                if arr is None:
                    return None
                return np.stack([arr[js, 0, :] for js, _ in per_w], axis=1)
            r = TimeEvolutionResult(p, gather(res.theta), gather(res.current), gather(res.voltage))
            r.node_solves_on_device = getattr(res, "node_solves_on_device", False)
            out.append(r)
        return out

    def simulations(self, seed=None, **options):
        """One GpuSimulation per part (each on its own stream), over the parts' union problems;
        ``options`` as for GpuSimulation. The parts draw noise from distinct Philox streams."""
        from .backend import GpuSimulation, _torch
        if options.get("device") is None:   # the caller's device, not each new thread's default
            options = dict(options, device=_torch().cuda.current_device())
        if self.Nj >= ONE_LANE_FROM_JUNCTIONS and not (options.get("tuning") or {}).get("pack_lanes"):
            # the parts' concurrent levels already hold many warps: one lane per packed supernode
            options = dict(options, tuning=dict(options.get("tuning") or {}, pack_lanes=1))
        sims = [None] * len(self.parts)

        def build(k):      # the parts' factorisations and plan uploads run in parallel host threads
            s = None if seed is None else (int(seed) + _SEED_STRIDE * k) % (1 << 63)
            sims[k] = GpuSimulation(self.parts[k].union_problem(), seed=s, **options)

        _in_threads([functools.partial(build, k) for k in range(len(self.parts))])
        return sims

    @staticmethod
    def run_simulations(sims, nsteps, use_graph=True):
        """Advance every part's simulation by nsteps steps, each from its own host thread: a long
        run blocks its caller while the GPU drains the queued graph launches, so one thread per
        part keeps all parts' launch chains queued together."""
        _in_threads([lambda s=s: s.run(nsteps, use_graph=use_graph) for s in sims])

    def compute(self, **options):
        """Step all problems; returns one TimeEvolutionResult per input problem. With several
        parts, each part's core runs in its own host thread, so their launch chains overlap."""
        if len(self.parts) == 1:
            return self._split(time_evolution(self.union_problem(), **options))
        if "core" in options:            # a replacement core (tests): the parts one after another
            results = [part._split(time_evolution(part.union_problem(), **options)) for part in self.parts]
        else:
            from .backend import time_evolution_core
            opts = dict(options)
            use_graph = opts.pop("use_graph", True)
            sims = self.simulations(**opts)
            results = [None] * len(sims)

            def work(k):
                core = functools.partial(time_evolution_core, sim=sims[k], use_graph=use_graph)
                results[k] = self.parts[k]._split(time_evolution(sims[k].problem, core=core))

            _in_threads([functools.partial(work, k) for k in range(len(sims))])
            for r in results:
                for x in r:
                    x.node_solves_on_device = True
        out = [None] * len(self.problems)
        for members, res in zip(self.part_members, results):
            for i, r in zip(members, res):
                out[i] = r
        return out
