"""Seeded synthetic workloads with the reference's shapes and distributions.

The reference has no public benchmark for this path; its random-obstacle
experiments (apps/CommonFunctions.h:77-177) place boxes in a workspace sphere
and reject boxes that make the start configuration invalid.  These
generators produce the same kinds of scenes with fixed seeds:

* ``planar_2dof_workload``   planar_2dof, 4 AABBs in a 2 m disk, 65,536 configs
* ``xarm6_workload``         xarm6 capsules (r 0.05, gripper 0.1, ground from
                             link 2), 50 cubes of 0.05 m in a 1 m ball around
                             (0, 0, 0.267) rejected if they touch q = 0,
                             1,048,576 configs in [-pi, pi]^6
* ``spatial10_edge_workload`` spatial_10dof (r 0.03), 200 rotated boxes turned
                             into fcl world AABBs in a 1.2 m ball around the
                             spatial scenarios' WS_center (0, 0, 0.1), rejected
                             if they touch q = 0; 262,144 edges discretised at
                             0.05 rad
* ``mixed_dof_workload``     spatial 14/18/22 (r 0.03), 500 AABBs in a 1.5 m
                             ball around WS_center, rejected if they touch
                             q = 0; 32,768/49,152/49,152 configs

Every array is float32 (the reference's State coordinates are
Eigen::VectorXf, include/state_spaces/State.h:27).
"""
import math
import os

import numpy as np

from . import robots as _robots
from ._abi import RPM_OBS_GROUND, RPM_OBS_DYNAMIC

MAX_DISTANCE = 1000.0


class Scene:
    """An obstacle set as the hot path sees it: fcl world AABBs (n, 6) float32,
    min_dist_tol (n,) float32 and RPM_OBS_* flags (n,) uint8."""

    def __init__(self, aabb, tol=None, flags=None, labels=None):
        self.aabb = np.ascontiguousarray(aabb, dtype=np.float32).reshape(-1, 6)
        n = self.aabb.shape[0]
        self.tol = (np.full(n, MAX_DISTANCE, np.float32) if tol is None
                    else np.ascontiguousarray(tol, dtype=np.float32))
        self.flags = np.zeros(n, np.uint8) if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
        self.labels = labels

    @property
    def n(self):
        return self.aabb.shape[0]


def box_aabb(dim, pos, quat_xyzw=(0.0, 0.0, 0.0, 1.0)):
    """fcl 0.7 world AABB of a box (src/environments/objects/Box.cpp:6-7):
    identity rotation -> (-dim/2) + pos .. dim/2 + pos, any other rotation ->
    the cube pos -/+ |dim/2|.  float32 arithmetic."""
    dim = np.asarray(dim, np.float32)
    pos = np.asarray(pos, np.float32)
    x, y, z, w = [np.float32(v) for v in quat_xyzw]
    h = np.float32(0.5) * dim
    if x == 0 and y == 0 and z == 0 and abs(w) == 1:
        return np.concatenate([(-h) + pos, h + pos]).astype(np.float32)
    rad = np.sqrt(h[0] * h[0] + (h[1] * h[1] + h[2] * h[2])).astype(np.float32)
    return np.concatenate([pos - rad, pos + rad]).astype(np.float32)


def ground_box():
    """The 'ground' obstacle of the xarm6 scenarios (data/xarm6/scenario1/scenario1.yaml:2-6)."""
    return box_aabb([1.5, 1.5, 0.1], [0.0, 0.0, -0.05]), np.float32(0.05)


def _ball(rng, n, center, radius):
    pts = []
    while len(pts) < n:
        p = rng.uniform(-1.0, 1.0, 3)
        if p @ p <= 1.0:
            pts.append(np.asarray(center) + radius * p)
    return np.array(pts)


def _seg_aabb_dist(a, b, box, samples=65):
    t = np.linspace(0.0, 1.0, samples)[:, None]
    p = a[None, :] + t * (b - a)[None, :]
    d = np.maximum(np.maximum(box[:3] - p, p - box[3:]), 0.0)
    return float(np.sqrt((d * d).sum(1)).min()), float(np.linalg.norm(b - a)) / (samples - 1)


def touches(robot, q, box, margin=0.01):
    """Conservative host test: True if the capsule skeleton at q comes within
    radius + margin of the box (used to reject obstacles at q = 0)."""
    sk = robot.skeleton_np(q)
    r = robot.capsule_radius
    for i in range(robot.num_links):
        d, h = _seg_aabb_dist(sk[i], sk[i + 1], box.astype(np.float64))
        if d <= r[i] + margin + h:
            return True
    return False


def uniform_configs(rng, n, dofs, lo=-math.pi, hi=math.pi):
    return rng.uniform(lo, hi, (n, dofs)).astype(np.float32)


def planar_2dof_workload(num_configs=65536, seed=0):
    rng = np.random.default_rng(seed)
    robot = _robots.planar_2dof(radius=0.0)
    boxes = []
    for _ in range(4):
        dx, dy = rng.uniform(0.1, 0.5, 2)
        rr, th = 2.0 * math.sqrt(rng.uniform()), rng.uniform(0, 2 * math.pi)
        boxes.append(box_aabb([dx, dy, 0.1], [rr * math.cos(th), rr * math.sin(th), 0.0]))
    scene = Scene(np.array(boxes))
    q = uniform_configs(rng, num_configs, 2)
    return robot, scene, q


def xarm6_workload(num_configs=1 << 20, num_obstacles=50, seed=1, gripper_length=0.1, radius=0.05):
    rng = np.random.default_rng(seed)
    robot = _robots.xarm6(radius=radius, gripper_length=gripper_length, ground_included=2)
    g_aabb, g_tol = ground_box()
    aabb = [g_aabb]
    tol = [g_tol]
    flags = [RPM_OBS_GROUND]
    q0 = np.zeros(6)
    while len(aabb) < num_obstacles + 1:
        c = _ball(rng, 1, (0.0, 0.0, 0.267), 1.0)[0]
        box = box_aabb([0.05, 0.05, 0.05], c)
        if touches(robot, q0, box):
            continue
        aabb.append(box)
        tol.append(np.float32(MAX_DISTANCE))
        flags.append(0)
    scene = Scene(np.array(aabb), np.array(tol, np.float32), np.array(flags, np.uint8))
    q = uniform_configs(rng, num_configs, 6)
    return robot, scene, q


SPATIAL_WS_CENTER = (0.0, 0.0, 0.1)   # WS_center of the spatial scenarios (data/spatial_10dof/*/*.yaml)


def random_obb_scene(rng, n, dim_lo, dim_hi, center, radius, rotated=True, reject_robot=None):
    """n boxes with dims U[dim_lo, dim_hi], centres uniform in a ball, as fcl
    world AABBs.  Like the reference's generator (which drops obstacles that
    make the start configuration invalid), boxes touching reject_robot at
    q = 0 are redrawn."""
    boxes = []
    q0 = None if reject_robot is None else np.zeros(reject_robot.num_dofs)
    while len(boxes) < n:
        dim = rng.uniform(dim_lo, dim_hi, 3)
        c = _ball(rng, 1, center, radius)[0]
        if rotated:
            qv = rng.normal(size=4)
            qv = qv / np.linalg.norm(qv)
        else:
            qv = np.array([0.0, 0.0, 0.0, 1.0])
        box = box_aabb(dim, c, qv)
        if q0 is not None and touches(reject_robot, q0, box):
            continue
        boxes.append(box)
    return Scene(np.array(boxes))


def spatial10_edge_workload(num_edges=1 << 18, seed=2, step=0.05):
    rng = np.random.default_rng(seed)
    robot = _robots.spatial(10, radius=0.03)
    scene = random_obb_scene(rng, 200, 0.02, 0.1, SPATIAL_WS_CENTER, 1.2, rotated=True, reject_robot=robot)
    q1 = uniform_configs(rng, num_edges, 10)
    u = rng.normal(size=(num_edges, 10))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    length = rng.uniform(0.01, 2.0, (num_edges, 1))
    q2 = (q1 + u * length).astype(np.float32)
    return robot, scene, q1, q2, np.float32(step)


def large_scene_workload(num_configs=65536, seed=6, num_obstacles=1000, dofs=22):
    """A spatial chain against a large obstacle set: boxes with dims U[0.02, 0.15] m,
    centres uniform in a 1.5 m ball (no rejection), configurations uniform in limits."""
    rng = np.random.default_rng(seed)
    robot = _robots.spatial(dofs, radius=0.03)
    boxes = [box_aabb(rng.uniform(0.02, 0.15, 3), c) for c in _ball(rng, num_obstacles, SPATIAL_WS_CENTER, 1.5)]
    return robot, Scene(np.array(boxes)), uniform_configs(rng, num_configs, dofs)


def mixed_dof_workload(counts=(32768, 49152, 49152), seed=3):
    rng = np.random.default_rng(seed)
    scene = random_obb_scene(rng, 500, 0.02, 0.15, SPATIAL_WS_CENTER, 1.5, rotated=False,
                             reject_robot=_robots.spatial(22, radius=0.03))
    parts = []
    for dofs, n in zip((14, 18, 22), counts):
        robot = _robots.spatial(dofs, radius=0.03)
        parts.append((robot, uniform_configs(rng, n, dofs)))
    return scene, parts


# ------------------------------------------------------------ scene I/O --
def load_scenario(path):
    """A scenario YAML of the reference (Environment.cpp:13-109), read by the
    library's rpm_scenario_read.  Returns (info, Scene): info is a dict of the
    robot fields (type, num_dofs, ground_included, capsules_radius,
    gripper_length, ws_center, ws_radius, q_start, q_goal)."""
    import ctypes
    from . import _abi
    from .engine import _check, load
    lib = load()
    info = _abi.ScenarioInfo()
    _check(lib.rpm_scenario_read(os.fsencode(path), ctypes.byref(info), None, None, None, 0))
    n = info.num_obstacles
    aabb = np.zeros((max(n, 1), 6), np.float32)
    tol = np.zeros(max(n, 1), np.float32)
    flags = np.zeros(max(n, 1), np.uint8)
    _check(lib.rpm_scenario_read(os.fsencode(path), ctypes.byref(info), aabb.ctypes.data, tol.ctypes.data,
                                 flags.ctypes.data, n))
    D = info.num_dofs
    out = {"type": info.type.decode(), "num_dofs": D, "ground_included": info.ground_included,
           "capsules_radius": np.array(info.capsules_radius[:info.num_radii], np.float32),
           "gripper_length": float(info.gripper_length), "ws_center": np.array(info.ws_center[:], np.float32),
           "ws_radius": float(info.ws_radius), "q_start": np.array(info.q_start[:D], np.float32),
           "q_goal": np.array(info.q_goal[:D], np.float32)}
    return out, Scene(aabb[:n], tol[:n], flags[:n])


def robot_of_scenario(info):
    """The robot a scenario names, with its capsule radii, gripper and ground rule."""
    name = info["type"]
    radius = info["capsules_radius"] if info["capsules_radius"].size else None
    kw = {} if radius is None else {"radius": radius}
    if name == "xarm6":
        return _robots.xarm6(gripper_length=info["gripper_length"], ground_included=info["ground_included"], **kw)
    rb = _robots.by_name(name, **kw)
    rb.set_ground_included(info["ground_included"])
    return rb


def load_random_scenario(path, num_obstacles, run, num_dofs, obstacle_dim):
    """One run of random_scenarios.yaml (apps/test_drgbt_random_obstacles.cpp:125-151):
    start, goal, the objects' positions and velocities, and the objects as a
    Scene of "dynamic_obstacle" boxes of obstacle_dim (identity rotation)."""
    from .engine import _check, load
    lib = load()
    start = np.zeros(num_dofs, np.float32)
    goal = np.zeros(num_dofs, np.float32)
    pos = np.zeros((max(num_obstacles, 1), 3), np.float32)
    vel = np.zeros((max(num_obstacles, 1), 3), np.float32)
    _check(lib.rpm_random_scenario_read(os.fsencode(path), int(num_obstacles), int(run), int(num_dofs),
                                        start.ctypes.data, goal.ctypes.data, pos.ctypes.data, vel.ctypes.data))
    pos, vel = pos[:num_obstacles], vel[:num_obstacles]
    boxes = np.array([box_aabb(obstacle_dim, p) for p in pos], np.float32).reshape(-1, 6)
    flags = np.full(num_obstacles, RPM_OBS_DYNAMIC, np.uint8)
    return start, goal, pos, vel, Scene(boxes, flags=flags)
