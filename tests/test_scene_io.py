"""Scene I/O: scenario YAML and random_scenarios.yaml readers of the C library
(host code, no GPU) against hand-written fixtures in the reference's format,
and, where the reference's data tree is present, over all its scenario files."""
import glob
import os
import re

import numpy as np
import pytest

from rpmplv2_gb300 import _abi, scenes

HERE = os.path.dirname(os.path.abspath(__file__))
SC = os.path.join(HERE, "golden", "scenarios")


@pytest.fixture(scope="module", autouse=True)
def built():
    from rpmplv2_gb300 import build
    build.build()


def test_xarm6_scenario_fields_and_obstacles():
    info, sc = scenes.load_scenario(os.path.join(SC, "xarm6_pillars.yaml"))
    assert info["type"] == "xarm6" and info["num_dofs"] == 6 and info["ground_included"] == 2
    assert np.allclose(info["capsules_radius"], [0.05, 0.11, 0.1, 0.08, 0.05, 0.05])
    assert info["gripper_length"] == np.float32(0.12) and info["ws_radius"] == np.float32(1.4)
    assert np.array_equal(info["q_goal"], np.array([2.5, 0.5, -2.0, 1.5, 0, 3.0], np.float32))
    # ground, two pillars, the moving box; the sphere is skipped
    assert sc.n == 4
    assert np.array_equal(sc.aabb[0], scenes.box_aabb([1.5, 1.5, 0.1], [0, 0, -0.05]))
    assert np.array_equal(sc.aabb[1], scenes.box_aabb([0.3, 0.2, 0.9], [0.6, 0.4, 0.45]))
    assert np.array_equal(sc.aabb[2], scenes.box_aabb([0.25, 0.25, 0.7], [-0.5, 0.45, 0.35],
                                                      (0, 0, 0.3826834, 0.9238795)))
    assert list(sc.flags) == [_abi.RPM_OBS_GROUND, 0, 0, _abi.RPM_OBS_DYNAMIC]
    assert list(sc.tol) == [np.float32(0.05), 1000.0, 1000.0, np.float32(0.2)]
    rb = scenes.robot_of_scenario(info)
    assert rb.num_dofs == 6 and rb.desc.ground_included == 2


def test_ground_left_out_without_ground_rule():
    """Environment.cpp:31-32: the ground is not added when ground_included is 0;
    "-   box:" items with wider indentation parse the same."""
    info, sc = scenes.load_scenario(os.path.join(SC, "spatial_no_ground.yaml"))
    assert info["ground_included"] == 0 and sc.n == 1
    assert np.array_equal(sc.aabb[0], scenes.box_aabb([0.2, 0.2, 0.2], [0.5, 0.0, 0.8]))
    rb = scenes.robot_of_scenario(info)
    assert rb.num_dofs == 14 and np.all(rb.capsule_radius == np.float32(0.03))


def test_random_scenario_runs():
    path = os.path.join(SC, "random_runs.yaml")
    start, goal, pos, vel, sc = scenes.load_random_scenario(path, 2, 1, 2, [0.2, 0.2, 0.2])
    assert np.array_equal(start, [1.0, 1.0]) and np.array_equal(goal, [-1.0, -1.0])
    assert np.array_equal(pos, np.float32([[1.5, 0, 0], [0, -1.5, 0]]))
    assert np.array_equal(vel, np.float32([[-0.3, 0, 0], [0, 0.3, 0]]))
    assert sc.n == 2 and np.all(sc.flags == _abi.RPM_OBS_DYNAMIC)
    assert np.array_equal(sc.aabb[0], scenes.box_aabb([0.2, 0.2, 0.2], [1.5, 0, 0]))
    s3 = scenes.load_random_scenario(path, 1, 0, 2, [0.2, 0.2, 0.2])
    assert np.array_equal(s3[1], [3.0, 0.0])
    from rpmplv2_gb300.engine import RpmError
    with pytest.raises(RpmError):
        scenes.load_random_scenario(path, 2, 7, 2, [0.2, 0.2, 0.2])   # no such run


def test_malformed_files_fail_loudly(tmp_path):
    from rpmplv2_gb300.engine import RpmError
    bad = tmp_path / "bad.yaml"
    bad.write_text("environment:\n  - cylinder:\n      dim: [1, 1, 1]\nrobot:\n  type: \"xarm6\"\n")
    with pytest.raises(RpmError):
        scenes.load_scenario(str(bad))
    bad.write_text("robot:\n  type: x\n    num_DOFs: 3\n")
    with pytest.raises(RpmError):
        scenes.load_scenario(str(bad))
    with pytest.raises(RpmError):
        scenes.load_scenario(str(tmp_path / "missing.yaml"))


def _reference_data():
    from oracle import build as ob
    root = os.path.join(ob.REF_ROOT, "data")
    return root if os.path.isdir(root) else None


def test_every_reference_scenario_reads():
    """Every scenario file of the reference's data tree reads, with as many boxes
    as its text lists (minus the ground where the ground rule is off)."""
    root = _reference_data()
    if root is None:
        pytest.skip("the reference's data tree is not present")
    n_files = 0
    for path in sorted(glob.glob(os.path.join(root, "*", "*", "*.yaml"))):
        text = open(path).read()
        if "environment:" not in text or "robot:" not in text:
            continue
        info, sc = scenes.load_scenario(path)
        boxes = len(re.findall(r"^\s*-\s*box\s*:", text, re.M))
        grounds = len(re.findall(r"label:\s*[\"']ground[\"']", text))
        want = boxes - (grounds if info["ground_included"] == 0 else 0)
        assert sc.n == want, path
        assert info["num_dofs"] > 0, path
        n_files += 1
    assert n_files >= 10
    for path in sorted(glob.glob(os.path.join(root, "*", "scenario_random_obstacles", "random_scenarios.yaml"))):
        m = re.search(r"^scenario_(\d+):", open(path).read(), re.M)
        k = int(m.group(1))
        D = len(re.search(r"start:\s*\[([^\]]*)\]", open(path).read()).group(1).split(","))
        start, goal, pos, vel, sc = scenes.load_random_scenario(path, k, 0, D, [0.1, 0.1, 0.1])
        assert start.shape == (D,) and pos.shape == (k, 3) and sc.n == k
