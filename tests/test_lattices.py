"""Lattice builders reproduce the reference's cycle matrix, numbering and current_base exactly."""
import numpy as np
import pytest
import scipy.sparse

import golden_cases as gc
from pyjjasim_gb300.circuit import HoneycombArray, SquareArray, TriangularArray

LAT = np.load(gc.GOLDEN + "/lattices.npz")
KEYS = sorted(set(k.split("__")[0] for k in LAT.files))
CLS = {"square": SquareArray, "honeycomb": HoneycombArray, "triangular": TriangularArray}


@pytest.mark.parametrize("key", KEYS)
def test_lattice_matches_reference(key):
    kind, size = key.split("_")
    nx, ny = map(int, size.split("x"))
    c = CLS[kind](nx, ny)
    z = {k.split("__")[1]: LAT[k] for k in LAT.files if k.startswith(key + "__")}
    A_ref = scipy.sparse.csr_matrix((z["A_data"], z["A_indices"], z["A_indptr"]), shape=tuple(z["A_shape"]))
    A = c.get_cycle_matrix().tocsr()
    assert A.shape == A_ref.shape
    assert (A != A_ref).nnz == 0
    M_ref = scipy.sparse.csr_matrix((z["M_data"], z["M_indices"], z["M_indptr"]), shape=tuple(z["M_shape"]))
    assert (c.get_cut_matrix().tocsr() != M_ref).nnz == 0
    assert np.array_equal(c.node_x, z["node_x"]) and np.array_equal(c.node_y, z["node_y"])
    assert np.array_equal(c.node1, z["node1"]) and np.array_equal(c.node2, z["node2"])
    for ang, k in ((0.0, "cb0"), (np.pi / 2, "cb90"), (np.pi / 6, "cb30")):
        np.testing.assert_allclose(c.current_base(ang), z[k], rtol=0, atol=1e-12)


def test_kirchhoff_structure():
    # every junction lies on at most two faces, and A M^T = 0 (faces are closed cycles)
    for c in (SquareArray(9, 7), HoneycombArray(4, 5), TriangularArray(6, 5)):
        A = c.get_cycle_matrix()
        assert np.all(np.asarray(abs(A).sum(axis=0)).ravel() <= 2)
        assert abs(A @ c.get_cut_matrix().T).max() == 0
