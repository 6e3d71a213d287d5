"""W = 1 packs: small supernodes of a level solved one per 1, 2 or 4 lanes (pack_lanes), 32,
16 or 8 of them per warp; with more than one lane a supernode's rows are split between its
lanes, and the backward sweep adds the lanes' partial sums with warp shuffles.

CPU: the schedule builds and passes its dataflow check for every lane count; other counts are
refused. GPU: W = 1 face solves against scipy's sparse direct solve (relative 1e-11) with packs
forced on every level (pack_min_warps = 1), in the level and cooperative schedules.
"""
import numpy as np
import pytest
import scipy.sparse.linalg

from pyjjasim_gb300 import backend
from pyjjasim_gb300 import _native as N
from pyjjasim_gb300 import plan as P
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_schedule_with_pack_lanes(lanes):
    f = P.get_factor(SquareArray(48, 48), 0.05, nd_leaf=8, ordering="nd")[0]
    n = f.check_schedule(1, {"pack_min_warps": 1, "pack_lanes": lanes})
    assert n[0] > 0 and n[1] > 0


def test_pack_lanes_values():
    f = P.get_factor(SquareArray(16, 16), 0.05, nd_leaf=8, ordering="nd")[0]
    with pytest.raises(N.JJAError):
        f.check_schedule(1, {"pack_min_warps": 1, "pack_lanes": 3})


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [1, 2, 4])
@pytest.mark.parametrize("lattice,n,ordering,schedule", [(SquareArray, 96, "nd", 1), (HoneycombArray, 40, "mmd", 1),
                                                         (TriangularArray, 48, "nd", 3)])
def test_packed_solve_matches_scipy(lattice, n, ordering, schedule, lanes):
    c = lattice(n, n)
    c.set_inductance(0.02)
    A, K = P.face_matrix(c, 0.05)
    b = np.random.default_rng(n + lanes).standard_normal(K.shape[0])
    x = backend.solve_faces(c, 0.05, b, ordering=ordering,
                            tuning={"pack_min_warps": 1, "pack_lanes": lanes, "schedule": schedule})
    ref = scipy.sparse.linalg.spsolve(K.tocsc(), b)
    assert float(np.abs(x - ref).max()) <= 1e-11 * float(np.abs(ref).max())
