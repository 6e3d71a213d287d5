"""Autotuner: search logic and cache on the CPU (a fake timing function), and on the GPU every
tuned launch shape gives the default's trajectory."""
import json

import numpy as np
import pytest

from pyjjasim_gb300 import autotune as AT
from pyjjasim_gb300.circuit import SquareArray


def test_coordinate_descent_finds_the_fastest_axis_values():
    # synthetic cost: rows_per_lane 4 and target_warps 152*8 help, relax (0, 0) hurts
    def measure(cfg):
        t = 1.0
        t *= 0.8 if cfg["rows_per_lane"] == 4 else 1.0
        t *= 0.9 if cfg["target_warps"] == 152 * 8 else 1.0
        t *= 1.3 if tuple(cfg["relax"]) == (0, 0.0) else 1.0
        t *= 0.99 if cfg["rhs_block"] == 16 else 1.0     # below the 2 % threshold: not taken
        return t

    best, t, log = AT.coordinate_descent(512, measure)
    assert best["rows_per_lane"] == 4 and best["target_warps"] == 152 * 8
    assert tuple(best["relax"]) == (-1, -1.0) and best["rhs_block"] == 0
    assert best["schedule"] == 1 and best["ordering"] == "auto" and best["groups"] == 0
    assert t == pytest.approx(0.72)
    cand = AT.candidates(512)
    n_tried = 1 + sum(int(np.prod([len(cand[n]) for n in (a if isinstance(a, tuple) else (a,))])) - 1
                      for a in AT.AXES)
    assert log[0][0] == AT.DEFAULT and len(log) == n_tried


def test_candidates_respect_the_batch_width():
    assert AT.candidates(1)["rhs_block"] == [0]          # one problem: one lane per problem only
    assert AT.candidates(8)["rhs_block"] == [0, 4, 2]
    assert AT.candidates(512)["rhs_block"] == [0, 16, 8]
    # subtree sizes: the library's rule first, none, then sizes that fit the subtree kernels
    for W in (1, 8, 17, 512):
        cand = AT.candidates(W)["subtree_rows"]
        assert cand[0] == 0 and -1 in cand and all(r <= 64 for r in cand)


def test_tuned_options_carry_every_solve_field():
    opts = AT.to_options(dict(AT.DEFAULT, subtree_rows=24, groups=3))
    assert opts["tuning"]["subtree_rows"] == 24 and opts["tuning"]["groups"] == 3
    from pyjjasim_gb300 import plan as P
    assert set(opts["tuning"]) <= set(P.TUNING_FIELDS)


def test_cache_is_written_and_reused(tmp_path, monkeypatch):
    monkeypatch.setenv(AT.CACHE_ENV, str(tmp_path / "tune.json"))
    c = SquareArray(6, 6)
    calls = []

    def measure(cfg):
        calls.append(cfg)
        return 2.0 if cfg["rows_per_lane"] == 4 else 3.0

    opts = AT.autotune(c, 0.05, 4, measure=measure, device_name="fake-gpu")
    assert opts["tuning"]["rows_per_lane"] == 4 and opts["relax"] == (-1, -1.0) and opts["ordering"] == "auto"
    n = len(calls)
    again = AT.autotune(c, 0.05, 4, measure=measure, device_name="fake-gpu")
    assert again == opts and len(calls) == n             # served from the cache
    data = json.loads((tmp_path / "tune.json").read_text())
    (key, entry), = data.items()
    assert key.startswith("fake-gpu|K=") and "W=4" in key
    assert entry["seconds_per_step"] == 2.0 and entry["default_seconds_per_step"] == 3.0
    # another W is another entry
    AT.autotune(c, 0.05, 5, measure=measure, device_name="fake-gpu")
    assert len(json.loads((tmp_path / "tune.json").read_text())) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("tuning,relax", [({"rows_per_lane": 2}, (-1, -1.0)), ({"rows_per_lane": 8}, (0, 0.0)),
                                          ({"rhs_block": 8, "target_warps": 152 * 64}, (64, 0.1)),
                                          ({"rhs_block": 2, "min_piece": 4, "target_warps": 152 * 200}, (-1, -1.0)),
                                          ({"schedule": 2}, (-1, -1.0)),
                                          ({"schedule": 2, "rows_per_lane": 8, "rhs_block": 4}, (0, 0.0)),
                                          ({"schedule": 2, "rows_per_lane": 2, "min_piece": 4,
                                            "target_warps": 152 * 200}, (64, 0.1)),
                                          ({"pdl": 1}, (-1, -1.0)),
                                          ({"groups": 1}, (-1, -1.0)),
                                          ({"pdl": 1, "schedule": 2, "rows_per_lane": 4}, (0, 0.0)),
                                          ({"subtree_rows": 24}, (-1, -1.0)), ({"subtree_rows": 64}, (0, 0.0)),
                                          ({"subtree_rows": 16, "rhs_block": 4}, (-1, -1.0))])
def test_tuned_launch_shapes_agree_with_default(tuning, relax):
    from pyjjasim_gb300 import TimeEvolutionProblem, backend
    c = SquareArray(20, 23)
    c.set_inductance(0.1)
    W = 16
    Is = c.current_base(0.0)[:, None, None] * np.linspace(0.3, 1.8, W)[None, :, None]
    prob = TimeEvolutionProblem(c, time_step=0.05, time_step_count=150, current_sources=Is, external_flux=0.2,
                                store_time_steps=[149])
    th0, _ = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps)
    th1, _ = backend.time_evolution_core(prob, prob.store_time_steps, prob.store_time_steps, tuning=tuning,
                                         relax=relax)
    scale = max(1.0, float(np.abs(th0).max()))
    assert float(np.abs(th1 - th0).max()) <= 1e-10 * scale


@pytest.mark.gpu
def test_autotune_on_gpu(tmp_path, monkeypatch):
    monkeypatch.setenv(AT.CACHE_ENV, str(tmp_path / "tune.json"))
    c = SquareArray(16, 16)
    opts = AT.autotune(c, 0.05, 32, steps=64)
    assert set(opts) == {"ordering", "relax", "tuning"}
    entry, = json.loads((tmp_path / "tune.json").read_text()).values()
    assert entry["seconds_per_step"] <= entry["default_seconds_per_step"]
