"""Failure detection without a GPU fault: a device-side wait that nothing can
satisfy runs out of its poll limit, the kernel reports the timeout through a
status word, the call returns RPM_ERR_TIMEOUT, and the context keeps working."""
import time

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import scenes

pytestmark = pytest.mark.gpu
RPM_ERR_TIMEOUT = -4


def test_bounded_wait_reports_timeout(engine):
    t0 = time.perf_counter()
    rc = engine.lib.rpm_probe_bounded_wait(engine.ctx, 256)
    assert rc == RPM_ERR_TIMEOUT
    assert b"gave up" in engine.lib.rpm_last_error_string()
    assert time.perf_counter() - t0 < 5.0
    assert engine.lib.rpm_probe_bounded_wait(engine.ctx, 0) == -1          # invalid limit
    # the context is still usable: a normal check gives the oracle's answer
    robot, scene, q = scenes.xarm6_workload(4096, seed=98)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
    engine.check_configs(sid, torch.from_numpy(q).cuda(), "fp32_ref", v, None, None)
    engine.sync()
    rv, _, _ = O.check_configs(robot, scene, q, prec="ref32", want=("valid",))
    assert np.array_equal(v.cpu().numpy(), rv)
    engine.destroy_scene(sid)
