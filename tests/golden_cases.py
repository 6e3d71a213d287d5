"""Rebuild the problems stored in tests/golden/*.npz (written by tests/golden/make_golden.py)."""
import glob
import os

import numpy as np
import scipy.sparse

from pyjjasim_gb300.circuit import Circuit
from pyjjasim_gb300.problem import TimeEvolutionProblem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "c*.npz")))


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def sparse(z, prefix):
    return scipy.sparse.csr_matrix((z[prefix + "_data"], z[prefix + "_indices"], z[prefix + "_indptr"]),
                                   shape=tuple(z[prefix + "_shape"]))


def circuit(z):
    L = sparse(z, "L").tocoo()
    # the fixtures were built with scalar self-inductance except the mutual-inductance case;
    # pass the same form back so the circuit's has-inductance flag matches the reference's
    diagonal_only = bool(np.all(L.row == L.col))
    Lin = sparse(z, "L").diagonal() if diagonal_only else sparse(z, "L").tocsc()
    return Circuit(sparse(z, "A"), critical_current=z["Ic"], resistance=z["R"], capacitance=z["C"],
                   inductance=Lin, cut_matrix=sparse(z, "M"), node_x=z["node_x"], node_y=z["node_y"],
                   node1=z["node1"], node2=z["node2"])


def problem(z, **over):
    c = circuit(z)
    dt = float(z["dt"])
    kw = dict(time_step=dt, time_step_count=int(z["Nt"]), stencil_width=int(z["stencil_width"]),
              store_time_steps=z["store_mask"])
    for key, arg in (("f", "external_flux"), ("Is", "current_sources"), ("Vs", "voltage_sources"),
                     ("T", "temperature")):
        if "in_" + key in z:
            kw[arg] = z["in_" + key]
    if "Is_spec_base" in z:
        base, dc, ac, fr = z["Is_spec_base"], float(z["Is_spec_dc"]), float(z["Is_spec_ac"]), float(z["Is_spec_freq"])
        kw["current_sources"] = lambda i: (base * (dc + ac * np.sin(2 * np.pi * fr * i * dt)))[:, None]
    for key, arg in (("th_m1", "config_at_minus_1"), ("th_m2", "config_at_minus_2"),
                     ("th_m3", "config_at_minus_3"), ("th_m4", "config_at_minus_4")):
        if "in_" + key in z:
            kw[arg] = z["in_" + key]
    kw.update(over)
    return TimeEvolutionProblem(c, **kw)


def seed(z):
    s = int(z["seed"])
    return None if s < 0 else s
