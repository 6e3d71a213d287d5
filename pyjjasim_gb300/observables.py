"""Node-space solves of the result observables on the GPU.

Node phases and potentials (pyjjasim time_evolution.py:692-714, 910-937) solve
M_r M_r^T x = M_r y with the last node grounded (M the cut matrix, M_r without its last row;
``Circuit.Msq_solve``, josephson_circuit.py:93-109) for every stored step and problem. On a
128x128 array with 512 problems that is 0.85 s per step with SuperLU on the host. Here the
same supernodal factorisation and triangular-solve kernels as the time step serve it:
M_r M_r^T is the face matrix K = A (L + diag(1/(Cv + Rv))) A^T of a circuit whose cycle matrix
is M_r, with R = 1, C = 0, L = 0 and dt = 1 (then 1/(Cv + Rv) = 1 exactly).
"""
import numpy as np

from .circuit import Circuit

_NODE_CIRCUITS = {}


class _NodeSpace(Circuit):
    """The reduced cut matrix as the cycle matrix of a circuit; its 'faces' are the nodes but
    the last, located at the node coordinates (which seed the nested-dissection ordering)."""

    def __init__(self, circuit):
        Mr = circuit.get_cut_matrix()[:-1, :]
        super().__init__(Mr, critical_current=1.0, resistance=1.0, capacitance=0.0, inductance=0.0)
        x, y = circuit.get_node_coordinates()
        self._xy = None if x is None else (np.asarray(x, np.float64)[:-1], np.asarray(y, np.float64)[:-1])

    def get_face_centroids(self):
        if self._xy is None:
            raise ValueError("no node coordinates")
        return self._xy


def _node_circuit(circuit):
    key = (id(circuit), getattr(circuit, "_version", 0))
    nc = _NODE_CIRCUITS.get(key)
    if nc is None or nc[0] is not circuit:
        nc = (circuit, _NodeSpace(circuit))
        _NODE_CIRCUITS.clear()          # one circuit at a time: results are read one after another
        _NODE_CIRCUITS[key] = nc
    return nc[1]


def msq_solve(circuit, b):
    """x with M_r M_r^T x[:-1] = b[:-1] and x[-1] = 0, for b of shape (Nn,) or (Nn, W), solved on
    the GPU (the host counterpart is ``Circuit.Msq_solve``)."""
    from .backend import solve_faces
    b = np.asarray(b, dtype=np.float64)
    x = solve_faces(_node_circuit(circuit), 1.0, b[:-1, ...])
    return np.append(x, np.zeros(b[-1:, ...].shape), axis=0)
