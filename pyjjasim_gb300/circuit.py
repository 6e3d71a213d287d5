"""Circuit description consumed by the GB300 time-evolution path.

The time-stepping core needs, from a circuit, only: the face cycle matrix A (Nf x Nj,
entries +-1), the junction vectors Ic, R, C and the inductance matrix L. This module
provides a minimal ``Circuit`` exposing exactly the accessor names the reference's core
reads (pyjjasim josephson_circuit.py: ``get_cycle_matrix`` :616, ``_Ic/_R/_C/_L``
:701-711, ``_Nj/_Nf`` :695-699, ``_has_inductance`` :807, ``get_inductance`` :582),
so either this class or a reference ``Circuit`` can be handed to the GPU backend.

It also builds the square, honeycomb and triangular lattices with the reference's
node, junction and face numbering (josephson_circuit.py:952-998, embedded_graph.py:
1093-1166), because the face order fixes the row order of A and therefore the
results' layout. Faces are found here by a planar face walk (each directed edge is
followed by the next edge clockwise around its head node, which keeps the face on the
left); faces with non-positive signed area are the outer boundary and are dropped, and
the remaining faces are ordered the way the reference enumerates them: by cycle length,
then by the smallest directed-edge id on the cycle, where edge ids count edges sorted
by (lower node, higher node) and a directed id is offset by Nj when the edge is walked
from its higher to its lower node. A_fj = +1 when face f walks junction j from its
node1 to its node2, -1 when it walks it backwards.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import scipy.sparse.csgraph


def _junction_vector(x, N, name):
    try:
        return np.broadcast_to(np.asarray(x, dtype=np.float64), (N,)).copy()
    except ValueError:
        raise ValueError(f"{name} must be scalar or array of length equal to junction count")


def _inductance_matrix(L, N):
    """Returns (L as sparse CSC, has_inductance flag); mirrors josephson_circuit.py:595-604, 727-756.

    A scalar or (Nj,) inductance becomes a diagonal matrix and the flag is "any entry
    nonzero". For an (Nj, Nj) matrix the reference stores the matrix's *is-zero* test in
    the has-inductance slot (set_inductance unpacks the third return value of
    _prepare_inducance_matrix, which is ``is_zero`` for 2-D input), so a nonzero mutual
    inductance matrix reports ``_has_inductance() == False`` and the voltage then omits
    the L dI/dt term (time_evolution.py:426-450). The flag is reproduced as-is so that
    results match the reference on the same inputs; the face-space matrix always uses L.
    """
    if scipy.sparse.issparse(L) or np.ndim(L) == 2:
        if L.shape != (N, N):
            raise ValueError("L must be scalar, (Nj,) array or (Nj, Nj) matrix")
        L = scipy.sparse.csc_matrix(L)
        if L.nnz and abs(L - L.T).max() > 1e-12 * max(1.0, abs(L).max()):
            raise ValueError("inductance matrix must be symmetric")
        is_zero = L.nnz == 0 or not np.any(L.data != 0)
        return L, bool(is_zero)
    x = _junction_vector(L, N, "L")
    if np.any(x < -10 * np.finfo(float).eps):
        raise ValueError("Inductance matrix not positive definite")
    return scipy.sparse.diags(x, 0).tocsc(), bool(np.any(x != 0.0))


class Circuit:
    """Minimal Josephson circuit: cycle matrix plus per-junction components.

    Parameters
    ----------
    cycle_matrix : (Nf, Nj) sparse matrix with entries +-1 (A).
    critical_current, resistance, capacitance : scalar or (Nj,) array.
    inductance : scalar, (Nj,) array, or (Nj, Nj) symmetric positive-definite matrix.
    cut_matrix : optional (Nn, Nj) node-junction incidence matrix (M), used by current_base.
    node_x, node_y, node1, node2 : optional geometry (used for face centroids).
    """

    def __init__(self, cycle_matrix, critical_current=1.0, resistance=1.0, capacitance=0.0,
                 inductance=0.0, cut_matrix=None, node_x=None, node_y=None, node1=None, node2=None):
        A = scipy.sparse.csc_matrix(cycle_matrix)
        self.cycle_matrix = A
        self.cut_matrix = None if cut_matrix is None else scipy.sparse.csc_matrix(cut_matrix)
        self.node_x, self.node_y = node_x, node_y
        self.node1, self.node2 = node1, node2
        self._version = 0
        self.set_critical_current(critical_current)
        self.set_resistance(resistance)
        self.set_capacitance(capacitance)
        self.set_inductance(inductance)
        self._Msq_factorized = None
        self._Asq_factorized = None

    # --- component setters (josephson_circuit.py:406-461, 595-604) -------------------------
    def set_critical_current(self, Ic):
        self.critical_current = _junction_vector(Ic, self._Nj(), "Ic")
        self._version += 1
        return self

    def set_resistance(self, R):
        R = _junction_vector(R, self._Nj(), "R")
        if np.any(R <= 0.0):
            raise ValueError("All junctions must have a positive resistor")
        self.resistance = R
        self._version += 1
        return self

    def set_capacitance(self, C):
        C = _junction_vector(C, self._Nj(), "C")
        if np.any(C < 0.0):
            raise ValueError("Capacitance cannot be negative.")
        self.capacitance = C
        self._version += 1
        return self

    def set_inductance(self, inductance):
        self.inductance, self._has_inductance_v = _inductance_matrix(inductance, self._Nj())
        self._version += 1
        return self

    # --- accessors read by the time-stepping core ------------------------------------------
    def get_cycle_matrix(self):
        return self.cycle_matrix

    def get_cut_matrix(self):
        if self.cut_matrix is None:
            raise ValueError("this circuit was built without a cut matrix")
        return self.cut_matrix

    def get_critical_current(self):
        return self.critical_current

    def get_resistance(self):
        return self.resistance

    def get_capacitance(self):
        return self.capacitance

    def get_inductance(self):
        return self.inductance

    def junction_count(self):
        return self._Nj()

    def face_count(self):
        return self._Nf()

    def node_count(self):
        return self._Nn()

    def _Nj(self):
        return self.cycle_matrix.shape[1]

    def _Nf(self):
        return self.cycle_matrix.shape[0]

    def _Nn(self):
        if self.cut_matrix is not None:
            return self.cut_matrix.shape[0]
        return 0 if self.node_x is None else len(self.node_x)

    def _Ic(self):
        return self.critical_current

    def _R(self):
        return self.resistance

    def _C(self):
        return self.capacitance

    def _L(self):
        return self.inductance

    def _has_inductance(self):
        return self._has_inductance_v

    def get_node_coordinates(self):
        return self.node_x, self.node_y

    def get_junction_nodes(self):
        return self.node1, self.node2

    def get_face_centroids(self):
        """Mean of each face's corner coordinates (used only to seed orderings)."""
        if self.node_x is None:
            raise ValueError("this circuit was built without node coordinates")
        A = self.cycle_matrix.tocsr()
        M = abs(A)
        # each face row touches its corner nodes twice through its junctions
        inc = scipy.sparse.csr_matrix((np.ones(2 * self._Nj()), (np.r_[self.node1, self.node2],
                                       np.r_[np.arange(self._Nj()), np.arange(self._Nj())])),
                                      shape=(len(self.node_x), self._Nj()))
        fn = (M @ inc.T).tocsr()
        fn.data[:] = 1.0
        cnt = np.asarray(fn.sum(axis=1)).ravel()
        return (fn @ self.node_x) / cnt, (fn @ self.node_y) / cnt

    # --- node-current helpers (static_problem.py:1174-1193, josephson_circuit.py:93-109) ----
    def Msq_solve(self, b):
        """Solves M_r M_r^T x = b[:-1] with the last node grounded (x[-1] = 0)."""
        if self._Msq_factorized is None:
            Mr = self.get_cut_matrix()[:-1, :]
            self._Msq_factorized = scipy.sparse.linalg.factorized((Mr @ Mr.T).tocsc())
        b = np.asarray(b, dtype=np.float64)
        return np.append(self._Msq_factorized(b[:-1, ...]), np.zeros(b[-1:, ...].shape), axis=0)

    def Asq_solve(self, b):
        """Solves A A^T x = b (A the cycle matrix; josephson_circuit.py:111-128)."""
        if self._Asq_factorized is None:
            A = self.get_cycle_matrix()
            self._Asq_factorized = scipy.sparse.linalg.factorized((A @ A.T).tocsc())
        return self._Asq_factorized(np.asarray(b, dtype=np.float64))

    def _has_capacitance(self):
        return bool(np.any(self.capacitance > 0))

    def node_to_junction_current(self, node_current):
        return -(self.get_cut_matrix().T @ self.Msq_solve(node_current))


# ------------------------------------------------------------------------------------------
# planar embedding -> faces
# ------------------------------------------------------------------------------------------

def _faces_from_embedding(x, y, n1, n2):
    """Cycle matrix A (Nf x Nj, CSC) of the bounded faces of a planar straight-line graph."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n1 = np.asarray(n1, np.int64)
    n2 = np.asarray(n2, np.int64)
    E = len(n1)
    lo, hi = np.minimum(n1, n2), np.maximum(n1, n2)
    order = np.lexsort((hi, lo))                 # sorted edge s <-> original junction order[s]
    rank = np.empty(E, np.int64)
    rank[order] = np.arange(E)
    # directed half-edges: h = 2*j + d, d=0 walks n1->n2, d=1 walks n2->n1
    tail = np.empty(2 * E, np.int64)
    head = np.empty(2 * E, np.int64)
    tail[0::2], head[0::2] = n1, n2
    tail[1::2], head[1::2] = n2, n1
    ang = np.arctan2(y[head] - y[tail], x[head] - x[tail])
    # out-going half-edges of every node sorted counter-clockwise by angle
    srt = np.lexsort((ang, tail))
    N = len(x)
    start = np.searchsorted(tail[srt], np.arange(N + 1))
    pos = np.empty(2 * E, np.int64)
    pos[srt] = np.arange(2 * E)
    twin = np.arange(2 * E) ^ 1
    # arriving along h at node v: next is the out-edge of v just clockwise of twin(h)
    t = twin
    v = tail[t]
    deg = start[v + 1] - start[v]
    p = pos[t] - start[v]
    nxt = srt[start[v] + (p - 1) % deg]
    # every cycle of the permutation h -> nxt[h] is one face boundary
    H = 2 * E
    perm_graph = scipy.sparse.csr_matrix((np.ones(H), (np.arange(H), nxt)), shape=(H, H))
    n_cyc, label = scipy.sparse.csgraph.connected_components(perm_graph, directed=True, connection="weak")
    area = 0.5 * np.bincount(label, weights=x[tail] * y[head] - x[head] * y[tail], minlength=n_cyc)
    length = np.bincount(label, minlength=n_cyc)
    j_all = np.arange(H) >> 1
    did = rank[j_all] + E * (tail != lo[j_all])   # directed id: offset when walked high -> low
    min_did = np.full(n_cyc, np.iinfo(np.int64).max)
    np.minimum.at(min_did, label, did)
    bounded = ~((area < 0) | np.isclose(area, 0.0))
    kept = np.flatnonzero(bounded)
    kept = kept[np.lexsort((min_did[kept], length[kept]))]
    row_of = np.full(n_cyc, -1)
    row_of[kept] = np.arange(len(kept))
    on_face = row_of[label] >= 0
    h = np.flatnonzero(on_face)
    vals = np.where((h & 1) == 0, 1.0, -1.0)
    A = scipy.sparse.csr_matrix((vals, (row_of[label[h]], h >> 1)), shape=(len(kept), E))
    return A.tocsc()


def _cut_matrix(n1, n2, N):
    E = len(n1)
    row = np.concatenate((n1, n2))
    col = np.concatenate((np.arange(E), np.arange(E)))
    data = np.concatenate((-np.ones(E), np.ones(E)))
    return scipy.sparse.coo_matrix((data, (row, col)), shape=(N, E)).tocsc()


class _Lattice(Circuit):
    def __init__(self, count_x, count_y, x_scale, y_scale, x, y, n1, n2):
        self.count_x, self.count_y = count_x, count_y
        self.x_scale, self.y_scale = x_scale, y_scale
        A = _faces_from_embedding(x, y, n1, n2)
        M = _cut_matrix(n1, n2, len(x))
        super().__init__(A, cut_matrix=M, node_x=np.asarray(x, float), node_y=np.asarray(y, float),
                         node1=np.asarray(n1), node2=np.asarray(n2))

    def current_base(self, angle, type="junction"):
        """Uniform current at ``angle`` (josephson_circuit.py:913-944)."""
        node = self._I_node_h() * np.cos(angle) + self._I_node_v() * np.sin(angle)
        if type == "node":
            return node
        return self.node_to_junction_current(node)


class SquareArray(_Lattice):
    """count_x x count_y nodes; junctions: all horizontal (row by row), then all vertical."""

    def __init__(self, count_x, count_y, x_scale=1.0, y_scale=1.0):
        gy, gx = np.mgrid[0:count_y, 0:count_x]
        idx = np.arange(count_x * count_y).reshape(count_y, count_x)
        n1 = np.concatenate((idx[:, :-1].ravel(), idx[:-1, :].ravel()))
        n2 = np.concatenate((idx[:, 1:].ravel(), idx[1:, :].ravel()))
        super().__init__(count_x, count_y, x_scale, y_scale, (gx * x_scale).ravel(), (gy * y_scale).ravel(), n1, n2)

    def _I_node_h(self):
        return (self.node_x == 0).astype(int) - np.isclose(self.node_x, (self.count_x - 1) * self.x_scale).astype(int)

    def _I_node_v(self):
        return (self.node_y == 0).astype(int) - np.isclose(self.node_y, (self.count_y - 1) * self.y_scale).astype(int)


class HoneycombArray(_Lattice):
    """Honeycomb lattice of count_x x count_y four-node unit cells."""

    def __init__(self, count_x, count_y, x_scale=1.0, y_scale=1.0):
        gy, gx = np.mgrid[0:count_y, 0:count_x]
        bx, by = 3.0 * gx, np.sqrt(3.0) * gy
        h = np.sqrt(0.75)
        x = np.concatenate((bx, bx + 0.5, bx + 1.5, bx + 2), axis=0).ravel()
        y = np.concatenate((by, by + h, by + h, by), axis=0).ravel()
        idx = np.arange(count_x * count_y).reshape(count_y, count_x)
        s = count_x * count_y
        a = (idx, idx[:-1, :] + s, idx + s, idx[:-1, :] + 2 * s, idx + 2 * s, idx[:, :-1] + 3 * s)
        b = (idx + s, idx[1:, :], idx + 2 * s, idx[1:, :] + 3 * s, idx + 3 * s, idx[:, 1:])
        n1 = np.concatenate([q.ravel() for q in a])
        n2 = np.concatenate([q.ravel() for q in b])
        super().__init__(count_x, count_y, x_scale, y_scale, x * x_scale, y * y_scale, n1, n2)

    def _I_node_h(self):
        n = self.count_y / (self.count_y - 0.5)
        return ((self.node_x == 0).astype(int) -
                np.isclose(self.node_x, (3 * self.count_x - 1) * self.x_scale).astype(int)) * n

    def _I_node_v(self):
        return ((self.node_y < 0.1 * np.sqrt(3) * self.y_scale).astype(int) -
                (self.node_y > (self.count_y - 0.6) * np.sqrt(3) * self.y_scale).astype(int)) * 1.5


class TriangularArray(_Lattice):
    """Triangular lattice of count_x x count_y two-node unit cells."""

    def __init__(self, count_x, count_y, x_scale=1.0, y_scale=1.0):
        gy, gx = np.mgrid[0:count_y, 0:count_x]
        bx, by = gx, np.sqrt(3.0) * gy
        x = np.concatenate((bx, bx + 0.5), axis=0)
        y = np.concatenate((by, by + np.sqrt(0.75)), axis=0)
        idx = np.arange(count_x * count_y).reshape(count_y, count_x)
        s = count_x * count_y
        a = (idx, idx[:, :-1], idx[:-1, :] + s, idx[:-1, :-1] + s, idx[:, :-1] + s, idx[:, 1:])
        b = (idx + s, idx[:, 1:], idx[1:, :], idx[1:, 1:], idx[:, 1:] + s, idx[:, :-1] + s)
        n1 = np.concatenate([q.ravel() for q in a])
        n2 = np.concatenate([q.ravel() for q in b])
        super().__init__(count_x, count_y, x_scale, y_scale, (x * x_scale).ravel(), (y * y_scale).ravel(), n1, n2)

    def _I_node_h(self):
        return ((self.node_x < 0.1 * self.x_scale).astype(int) -
                (self.node_x > (self.count_x - 0.6) * self.x_scale).astype(int)) * np.sqrt(3)

    def _I_node_v(self):
        return (self.node_y == 0).astype(int) - \
            np.isclose(self.node_y, (self.count_y - 0.5) * np.sqrt(3) * self.y_scale).astype(int)
