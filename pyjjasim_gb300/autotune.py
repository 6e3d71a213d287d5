"""Autotuner of the face-space solve: supernode amalgamation and the triangular-solve launch shape.

No counterpart in the reference (its solve is scipy's SuperLU). The cost of a time step on the
GPU depends on choices that have no single best value across array sizes and batch widths W:

* ``schedule``: one launch per elimination-tree level, one persistent dataflow launch per
  sweep whose work items wait on per-supernode completion counters, or one cooperative launch
  per sweep with grid-wide barriers between the levels (no launch gaps between levels);
* ``pdl``: programmatic dependent launch of the step's kernels (launch latency hidden behind
  the previous kernel's tail; pays off when the kernels are short);
* ``ordering``: nested dissection (shallow tree, big supernodes) or minimum degree (about 30 %
  less fill on 2-D arrays, but a deeper tree of smaller supernodes); ``"auto"`` (the library's
  default) picks by the step's size;
* ``groups``: the step's problems as independent groups on concurrent streams (each fills the
  SMs the other groups' level tails leave idle);
* ``relax``: how far supernodes are amalgamated (fewer, wider supernodes and fewer elimination-
  tree levels, i.e. fewer launches, against extra flops on explicit zeros);
* ``rows_per_lane`` (1, 2, 4, 8): output rows a lane accumulates per work item (more FMAs per load
  against fewer warps);
* ``rhs_block`` (a power of two <= 32): problems a warp handles side by side (the remaining
  lanes take more rows);
* ``target_warps``: how aggressively the few, long dot products at the top of the elimination
  tree are split into atomically accumulated pieces;
* ``subtree_rows``: how large the subtrees at the bottom of the tree are that are solved in
  shared memory in one launch per sweep (one warp per subtree from 32 problems per warp, packs of
  subtrees of one shape below; 0: the library's rule; -1: none).

``autotune`` times candidates with CUDA events on graph-replayed steps of a synthetic problem
on the same circuit, time step, stencil width and W (the step's cost does not depend on the
phase values), walking one axis at a time from the library defaults (coordinate descent), and
keeps the fastest in a JSON cache keyed by GPU name, face-space matrix and W. The result is a
dict of ``GpuSimulation`` / ``time_evolution_core`` options: ``{"relax": ..., "tuning": ...}``.
"""
import itertools
import json
import os
import tempfile

import numpy as np

from . import plan as P

CACHE_ENV = "PYJJASIM_GB300_TUNE_CACHE"
DEFAULT = {"schedule": 1, "ordering": "auto", "relax": (-1, -1.0), "rows_per_lane": 0, "rows_per_lane_fwd": 0,
           "rhs_block": 0, "target_warps": 0, "pdl": 0, "groups": 0, "subtree_rows": 0}
# searched in this order; a tuple is searched jointly (ordering and rows per lane interact:
# minimum degree's smaller supernodes want fewer rows per warp). Rows per lane 0 = the library's
# defaults (1, and 2 in the forward sweep from W = 256 on); a nonzero value sets both sweeps
# unless rows_per_lane_fwd sets the forward one.
AXES = (("ordering", "rows_per_lane"), "rows_per_lane_fwd", "schedule", "pdl", "groups", "rhs_block", "target_warps",
        "subtree_rows", "relax")


def cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "pyjjasim_gb300",
                                                     "tuning.json")


def default_rhs_block(W):
    wb = 1
    while wb < min(W, 32):
        wb <<= 1
    return wb


def candidates(W):
    """Values tried per axis (the first is the default)."""
    wb = default_rhs_block(W)
    return {
        "schedule": [1, 2, 3],
        "pdl": [0, 1],
        "ordering": ["auto", "nd", "mmd"],
        "groups": [0, 1, 2, 3, 4] if W >= 64 else [0],
        "rows_per_lane": [0, 1, 2, 4],
        "rows_per_lane_fwd": [0, 1, 2, 4],
        "rhs_block": [0] + [b for b in (wb // 2, wb // 4) if b >= 1],
        "target_warps": [0, 152 * 8, 152 * 24, 152 * 64],
        "subtree_rows": [0, -1, 24, 48] if W >= 17 else [0, -1, 16, 32],
        "relax": [(-1, -1.0), (0, 0.0), (64, 0.1)],
    }


def to_options(cfg):
    """GpuSimulation options of a configuration."""
    return {"ordering": str(cfg["ordering"]), "relax": tuple(cfg["relax"]),
            "tuning": {"rows_per_lane": int(cfg["rows_per_lane"]),
                       "rows_per_lane_fwd": int(cfg.get("rows_per_lane_fwd", 0)),
                       "rhs_block": int(cfg["rhs_block"]), "target_warps": int(cfg["target_warps"]),
                       "schedule": int(cfg["schedule"]), "pdl": int(cfg.get("pdl", 0)),
                       "groups": int(cfg.get("groups", 0)), "subtree_rows": int(cfg.get("subtree_rows", 0))}}


def coordinate_descent(W, measure, min_gain=0.02):
    """Walk AXES one at a time from DEFAULT, keeping a value when ``measure(cfg)`` (seconds per
    step) improves on the best so far by more than ``min_gain``. Returns (best, best time, log)."""
    best = dict(DEFAULT)
    best_t = measure(best)
    log = [(dict(best), best_t)]
    cand = candidates(W)
    for axis in AXES:
        names = axis if isinstance(axis, tuple) else (axis,)
        for values in itertools.product(*(cand[n] for n in names)):
            if all(best[n] == v for n, v in zip(names, values)):
                continue
            cfg = dict(best)
            cfg.update(zip(names, values))
            t = measure(cfg)
            log.append((dict(cfg), t))
            if t < best_t * (1.0 - min_gain):
                best, best_t = cfg, t
    return best, best_t, log


def _synthetic_problem(circuit, dt, W, stencil_width):
    from .problem import TimeEvolutionProblem
    Nj = circuit._Nj()
    rng = np.random.default_rng(0)
    th = rng.uniform(-np.pi, np.pi, (Nj, W))
    return TimeEvolutionProblem(circuit, time_step=dt, time_step_count=1, external_flux=np.full((1, W, 1), 0.1),
                                config_at_minus_1=th, config_at_minus_2=th, stencil_width=stencil_width)


def _gpu_measure(problem, steps, nd_leaf, device):
    from .backend import GpuSimulation

    def measure(cfg):
        import torch
        opts = to_options(cfg)
        sim = GpuSimulation(problem, noise="philox", seed=0, device=device, nd_leaf=nd_leaf,
                            ordering=opts["ordering"], relax=opts["relax"], tuning=opts["tuning"])
        G = 16 * (sim.width - 1)
        sim.run(G + 1, use_graph=True)           # capture the graph, warm the caches
        sim.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = max(steps, 2 * G)
        e0.record(sim.stream)
        sim.run(n, use_graph=True)
        e1.record(sim.stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / n

    return measure


def _load_cache(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(path, cache):
    d = os.path.dirname(path)
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, suffix=".tmp")
    with os.fdopen(fd, "w") as fh:
        json.dump(cache, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def cache_key(device_name, circuit, dt, W, stencil_width, nd_leaf=8):
    A, K = P.face_matrix(circuit, dt)
    return f"{device_name}|K={P._digest(K.indptr, K.indices, K.data)}|W={W}|width={stencil_width}|leaf={nd_leaf}"


def autotune(circuit, dt, W, stencil_width=3, nd_leaf=8, steps=64, use_cache=True, device=None, measure=None,
             device_name=None):
    """Options ({"ordering", "relax", "tuning"}) for the fastest step of W problems on ``circuit``.

    ``measure(cfg) -> seconds per step`` replaces the GPU timing (tests); ``use_cache=False``
    re-tunes and does not read the cache (the result is still stored)."""
    if device_name is None:
        import torch
        device_name = torch.cuda.get_device_name(device)
    key = cache_key(device_name, circuit, dt, W, stencil_width, nd_leaf)
    path = cache_path()
    cache = _load_cache(path)
    if use_cache and key in cache:
        return to_options(cache[key]["best"])
    if measure is None:
        measure = _gpu_measure(_synthetic_problem(circuit, dt, W, stencil_width), steps, nd_leaf, device)
    best, best_t, log = coordinate_descent(W, measure)
    cache = _load_cache(path)
    cache[key] = {"best": {k: (list(v) if isinstance(v, tuple) else v) for k, v in best.items()},
                  "seconds_per_step": best_t, "default_seconds_per_step": log[0][1],
                  "tried": [[{k: (list(v) if isinstance(v, tuple) else v) for k, v in c.items()}, t] for c, t in log]}
    _store_cache(path, cache)
    return to_options(best)
