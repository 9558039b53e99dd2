"""Scenario files into device scenes: a scenario read by rpm_scenario_read and
a random_scenarios run, uploaded and checked on the GPU against the oracle."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

pytestmark = pytest.mark.gpu
SC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scenarios")


def _check(engine, rb, sc, q):
    sid = engine.create_scene(engine.upload_robot(rb), sc)
    C = q.shape[0]
    v = torch.zeros(C, dtype=torch.uint8, device="cuda")
    d = torch.zeros(C, dtype=torch.float64, device="cuda")
    engine.check_configs(sid, torch.from_numpy(q).cuda(), "fp32_ref", v, d, None)
    engine.sync()
    rv, rd, _ = O.check_configs(rb, sc, q, prec="ref32", want=("valid", "dist"))
    assert np.array_equal(v.cpu().numpy(), rv)
    assert np.array_equal(d.cpu().numpy().view(np.uint64), rd.view(np.uint64))
    engine.destroy_scene(sid)
    return rv


def test_scenario_file_on_device(engine):
    info, sc = scenes.load_scenario(os.path.join(SC, "xarm6_pillars.yaml"))
    rb = scenes.robot_of_scenario(info)
    q = scenes.uniform_configs(np.random.default_rng(95), 4096, 6)
    q[0], q[1] = info["q_start"], info["q_goal"]
    rv = _check(engine, rb, sc, q)
    assert 0 < rv.sum() < rv.size


def test_random_scenario_on_device(engine):
    start, goal, pos, vel, sc = scenes.load_random_scenario(os.path.join(SC, "random_runs.yaml"), 2, 0, 2,
                                                           [0.3, 0.3, 0.3])
    rb = robots.planar_2dof(radius=0.0)
    q = scenes.uniform_configs(np.random.default_rng(96), 4096, 2)
    q[0], q[1] = start, goal
    _check(engine, rb, sc, q)
