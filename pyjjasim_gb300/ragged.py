"""Ragged batches: problems on different circuits stepped together in one launch sequence.

The reference batches W problems only when they share one circuit (the W axis of
``TimeEvolutionProblem``, time_evolution.py:20-116); different lattices need separate
``compute()`` calls. Here a batch of problems on different circuits (square, honeycomb,
triangular arrays of different sizes, each possibly with several problems) is stepped as ONE
system: the disjoint union of all (problem, w) copies of their circuits. Its cycle matrix and
face-space matrix are block diagonal, so one nested-dissection factorisation yields a forest
whose trees' levels are merged, and every time step is one sequence of level launches over all
problems at once, with the per-problem state laid out back to back (W = 1 in the union).

Restrictions: all problems share the time step, step count, stencil width and store mask
(``RaggedBatch`` raises otherwise), and use the default current-phase relation.
"""
import numpy as np
import scipy.sparse

from .circuit import Circuit
from .problem import TimeEvolutionProblem, TimeEvolutionResult, time_evolution

__all__ = ["RaggedBatch"]


def _geometry(c):
    x, y = c.get_node_coordinates()
    n1, n2 = c.get_junction_nodes()
    if x is None or n1 is None:
        raise ValueError("ragged batches need circuits with node coordinates and junction nodes")
    return np.asarray(x, float), np.asarray(y, float), np.asarray(n1), np.asarray(n2)


class RaggedBatch:
    """A list of TimeEvolutionProblems (any circuits) computed together on the GPU."""

    def __init__(self, problems):
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
        self._build_union()

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

    def compute(self, **options):
        """Step all problems together; returns one TimeEvolutionResult per input problem."""
        res = time_evolution(self.union_problem(), **options)
        out = []
        for p, per_w in zip(self.problems, self.slices):
            def gather(arr):
                if arr is None:
                    return None
                return np.stack([arr[js, 0, :] for js, _ in per_w], axis=1)
            out.append(TimeEvolutionResult(p, gather(res.theta), gather(res.current), gather(res.voltage)))
        return out
