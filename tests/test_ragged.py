"""Ragged batches (different lattices and sizes in one launch sequence).

CPU: the disjoint-union construction and the per-problem split, checked with the oracle as
the core against separate oracle runs of each problem. GPU: the same batch through the GPU
core against those separate oracle runs.
"""
import numpy as np
import pytest

from oracle import rcsj_oracle
from pyjjasim_gb300 import HoneycombArray, SquareArray, TimeEvolutionProblem, TriangularArray
from pyjjasim_gb300.ragged import RaggedBatch

NT = 150


def _problems():
    rng = np.random.default_rng(3)
    out = []
    specs = [(SquareArray(6, 5), 2, 0.1), (HoneycombArray(3, 3), 1, 0.23), (TriangularArray(4, 4), 3, 0.05),
             (SquareArray(9, 4), 1, 0.3)]
    for c, W, f in specs:
        c.set_capacitance(rng.uniform(0, 0.5))
        Is = c.current_base(0.2)[:, None, None] * np.linspace(0.3, 1.3, W)[None, :, None]
        th1 = 0.2 * rng.standard_normal((c.junction_count(), W))
        out.append(TimeEvolutionProblem(c, time_step=0.05, time_step_count=NT, current_sources=Is, external_flux=f,
                                        config_at_minus_1=th1, config_at_minus_2=th1 * 0.99,
                                        store_time_steps=np.arange(0, NT, 10)))
    return out


def _check(results, problems, rtol):
    for res, p in zip(results, problems):
        th, I, V = rcsj_oracle.time_evolution(p)
        for got, ref in ((res.get_theta(), th), (res.get_current(), I), (res.get_voltage(), V)):
            scale = max(1.0, float(np.abs(ref).max()))
            assert got.shape == ref.shape
            assert float(np.abs(got - ref).max()) <= rtol * scale
        assert np.array_equal(res.get_vortex_configuration(),
                              rcsj_oracle.vortex_configuration(p.get_circuit().get_cycle_matrix(), th))


@pytest.mark.parametrize("parts", [1, 2, 3])
def test_union_layout_with_oracle_core(parts):
    problems = _problems()
    batch = RaggedBatch(problems, parts=parts)
    assert len(batch.parts) == parts
    assert batch.Nj == sum(p.get_circuit()._Nj() * p.get_problem_count() for p in problems)
    assert batch.Nf == sum(p.get_circuit()._Nf() * p.get_problem_count() for p in problems)
    if parts > 1:   # every problem in exactly one part, the parts balanced by junction count
        assert sorted(i for m in batch.part_members for i in m) == list(range(len(problems)))
        with pytest.raises(ValueError):
            batch.union_problem()
    _check(batch.compute(core=rcsj_oracle.evolve), problems, rtol=1e-11)


def test_default_parts():
    from pyjjasim_gb300.ragged import default_parts
    assert len(RaggedBatch(_problems()).parts) == 1       # small batches stay one union
    # one part per ~2^19 junctions from 2^20 junctions on, 2 to 8 of them
    assert [default_parts(n) for n in (980588, 1 << 20, 1200000, 4530208, 30964399)] == [1, 2, 3, 8, 8]


def test_mismatched_problems_rejected():
    a, b = SquareArray(4, 4), SquareArray(5, 5)
    with pytest.raises(ValueError):
        RaggedBatch([TimeEvolutionProblem(a, time_step_count=10), TimeEvolutionProblem(b, time_step_count=11)])


@pytest.mark.gpu
@pytest.mark.parametrize("parts", [1, 2])
def test_ragged_batch_on_gpu(parts):
    problems = _problems()
    _check(RaggedBatch(problems, parts=parts).compute(), problems, rtol=1e-9)


@pytest.mark.gpu
def test_three_part_batch_of_all_lattices_against_the_oracle():
    """Six problems, square / honeycomb / triangular at sides 64-80 (about 140k junctions), run
    as three concurrent parts (each its own union, factor and stream); every problem against the
    oracle run alone: phases 1e-9 relative, vortex configurations equal."""
    Nt = 120
    specs = [(SquareArray, 64, 0.6), (HoneycombArray, 64, 1.1), (TriangularArray, 70, 0.9), (SquareArray, 80, 1.5),
             (HoneycombArray, 66, 0.4), (TriangularArray, 64, 1.3)]
    problems = []
    for cls, n, b in specs:
        c = cls(n, n)
        Is = c.current_base(0.0)[:, None, None] * np.array([b])[None, :, None]
        problems.append(TimeEvolutionProblem(c, time_step=0.05, time_step_count=Nt, current_sources=Is,
                                             external_flux=0.2, store_time_steps=[Nt // 2, Nt - 1],
                                             store_current=False, store_voltage=False))
    batch = RaggedBatch(problems, parts=3)
    assert len(batch.parts) == 3
    for res, p in zip(batch.compute(), problems):
        th, _, _ = rcsj_oracle.time_evolution(p)
        scale = max(1.0, float(np.abs(th).max()))
        assert float(np.abs(res.get_theta() - th).max()) <= 1e-9 * scale
        assert np.array_equal(res.get_vortex_configuration(),
                              rcsj_oracle.vortex_configuration(p.get_circuit().get_cycle_matrix(), th))
