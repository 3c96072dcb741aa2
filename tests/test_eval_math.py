"""The arithmetic behind the equal-time numbers (cpppt.guiding_eval,
cpppt.batch_guiding_eval), on CPU: relMSE, the log-log interpolation of
the time a method needs to reach a target error, and the config-5 scene
plan (seeded, triangle counts in range)."""
import math

import numpy as np
import pytest
import torch


def test_rel_mse():
    from cpppt.guiding_eval import rel_mse
    ref = torch.full((4, 4, 3), 0.1)
    x = ref + 0.1
    assert rel_mse(x, ref) == pytest.approx(0.01 / (0.01 + 0.01))
    assert rel_mse(ref, ref) == 0.0


def test_time_to_reach_interpolates_log_log():
    from cpppt.guiding_eval import time_to_reach
    rows = [(10.0, 100, 1e-2), (20.0, 200, 5e-3), (40.0, 400, 2.5e-3)]
    assert time_to_reach(rows, 1e-2) == 10.0
    # 1/t error curve: the target 7.07e-3 is reached at t = 10 sqrt(2)
    assert time_to_reach(rows, 1e-1 / (10 * math.sqrt(2))) == pytest.approx(10 * math.sqrt(2), rel=1e-9)
    assert time_to_reach(rows, 1e-3) is None
    assert time_to_reach(rows, 1.0) == 10.0  # already below at the first checkpoint


def test_config5_plan():
    from cpppt.batch_guiding_eval import plan
    p = plan(8, 5, 5e5, 4e6)
    assert p == plan(8, 5, 5e5, 4e6)
    assert [q["scene_seed"] for q in p] == list(range(5, 13))
    for q in p:
        tris = 12000 * q["box_subdiv"] ** 2 + 38
        assert 5e5 * 0.7 < tris < 4e6 * 1.3
