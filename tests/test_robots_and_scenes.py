"""Robot tables against the reference's URDFs, and the seeded workloads."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from rpmplv2_gb300 import robots, scenes

from oracle.build import REF_ROOT as REF   # the reference tree the oracle recipe reads (absent on GPU hosts)


def urdf_joints(name):
    path = os.path.join(REF, "data", name, name + ".urdf")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    out = []
    for j in ET.parse(path).getroot().findall("joint"):
        if j.get("type") != "revolute":
            continue
        o, a, lim = j.find("origin"), j.find("axis"), j.find("limit")
        out.append(([float(v) for v in o.get("xyz").split()], [float(v) for v in o.get("rpy").split()],
                    [float(v) for v in a.get("xyz").split()], (float(lim.get("lower")), float(lim.get("upper")))))
    return out


@pytest.mark.parametrize("name", ["planar_2dof", "planar_10dof", "spatial_10dof", "spatial_14dof", "spatial_18dof",
                                  "spatial_22dof", "xarm6"])
def test_tables_match_urdf(name):
    rb = robots.by_name(name)
    joints = urdf_joints(name)
    assert len(joints) == rb.num_dofs
    for k, (xyz, rpy, axis, lim) in enumerate(joints):
        assert np.allclose(rb.desc.origin_xyz[k][:], xyz)
        assert np.allclose(rb.desc.origin_rot[k][:], robots.rpy_to_matrix(*rpy))
        assert rb.desc.joint_axis[k] == int(np.argmax(np.abs(axis)))
        assert np.allclose(rb.limits[k], lim, atol=1e-6)


def test_rotations_are_orthonormal():
    for rpy in [(-1.5708, 0, 0), (1.5708, 0, 0), (0.3, -0.2, 1.1)]:
        M = np.array(robots.rpy_to_matrix(*rpy)).reshape(3, 3)
        assert np.allclose(M @ M.T, np.eye(3), atol=1e-15)


def test_workloads_are_seeded_and_shaped():
    r1, s1, q1 = scenes.xarm6_workload(1000, seed=9)
    r2, s2, q2 = scenes.xarm6_workload(1000, seed=9)
    assert np.array_equal(q1, q2) and np.array_equal(s1.aabb, s2.aabb)
    assert q1.dtype == np.float32 and q1.shape == (1000, 6) and s1.n == 51
    assert s1.flags[0] == 1 and s1.tol[0] == np.float32(0.05)
    # no obstacle touches the robot at q = 0
    for j in range(1, s1.n):
        assert not scenes.touches(r1, np.zeros(6), s1.aabb[j], margin=0.0)
    rb, sc, e1, e2, step = scenes.spatial10_edge_workload(100, seed=2)
    assert sc.n == 200 and e1.shape == (100, 10)
    L = np.linalg.norm(e2.astype(np.float64) - e1, axis=1)
    assert L.min() >= 0.0099 and L.max() <= 2.0001
    sc3, parts = scenes.mixed_dof_workload(counts=(10, 20, 30), seed=3)
    assert sc3.n == 500 and [p[1].shape for p in parts] == [(10, 14), (20, 18), (30, 22)]


@pytest.mark.parametrize("name,type_name", [("planar_2dof", "2dof"), ("planar_10dof", "10dof"), ("xarm6", "xarm6"),
                                            ("spatial_10dof", "spatial_10dof"), ("spatial_14dof", "spatial_14dof"),
                                            ("spatial_18dof", "spatial_18dof"), ("spatial_22dof", "spatial_22dof")])
def test_builtin_robot_tables_match(name, type_name):
    """rpm_robot_builtin (the C library's URDF tables, used by the C++ adapter
    to describe a robots::AbstractRobot by its getType()) equals the Python
    tables byte for byte once radii, ground rule and gripper are set alike."""
    import ctypes
    from rpmplv2_gb300 import _abi, engine, robots
    lib = engine.load()
    d = _abi.RobotDesc()
    assert lib.rpm_robot_builtin(type_name.encode(), ctypes.byref(d)) == 0
    r = robots.by_name(name) if name != "xarm6" else robots.xarm6(radius=0.0, gripper_length=0.0, ground_included=0)
    if name != "xarm6":
        r.set_capsule_radius(0.025)
    assert bytes(d) == bytes(r.desc)
    assert lib.rpm_robot_builtin(b"no_such_robot", ctypes.byref(d)) != 0
