"""Known-answer and property tests of the oracle (hand-solvable geometry)."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

BOX = np.array([0, 0, 0, 1, 1, 1], np.float32)


def test_planar_skeleton_kat():
    rb = robots.planar_2dof()
    sk = O.skeleton(rb, np.array([[0, 0], [math.pi / 2, 0], [0, math.pi / 2]], np.float32))
    assert np.allclose(sk[0], [[0, 0, 0], [1, 0, 0], [2, 0, 0]])
    assert np.allclose(sk[1], [[0, 0, 0], [0, 1, 0], [0, 2, 0]], atol=1e-7)
    assert np.allclose(sk[2], [[0, 0, 0], [1, 0, 0], [1, 1, 0]], atol=1e-7)


def test_xarm6_skeleton_matches_host_fk():
    rb = robots.xarm6(gripper_length=0.1)
    q = np.random.default_rng(0).uniform(-3, 3, (32, 6)).astype(np.float32)
    sk = O.skeleton(rb, q, prec="ref64")
    for k in range(32):
        assert np.allclose(sk[k], rb.skeleton_np(q[k]), atol=1e-12)
    sk0 = O.skeleton(rb, np.zeros((1, 6), np.float32))[0]
    assert np.allclose(sk0[0], 0) and np.allclose(sk0[1], [0, 0, 0.267])


@pytest.mark.parametrize("prec", ["ref32", "ref64"])
def test_distance_regions(prec):
    r = 0.1
    # face region: segment parallel to the top face at height 0.5
    d, _, _ = O.prim_distance([0.2, 0.3, 1.5], [0.7, 0.6, 1.5], r, BOX, prec)
    assert abs(d - (0.5 - r)) < 1e-6
    # edge region: segment beyond x max and z max, parallel to the y edge
    d, _, _ = O.prim_distance([1.3, 0.2, 1.4], [1.3, 0.8, 1.4], r, BOX, prec)
    assert abs(d - (math.hypot(0.3, 0.4) - r)) < 1e-6
    # vertex region: a short segment near the (1,1,1) corner
    d, _, _ = O.prim_distance([2, 2, 2], [2, 2, 3], r, BOX, prec)
    assert abs(d - (math.sqrt(3) - r)) < 1e-6
    # an endpoint inside the box: 0, radius not subtracted
    d, _, _ = O.prim_distance([0.5, 0.5, 0.5], [3, 3, 3], r, BOX, prec)
    assert d == 0.0
    # a segment piercing the box from outside: collision (d <= 0)
    d, _, _ = O.prim_distance([-1, 0.5, 0.5], [2, 0.5, 0.5], r, BOX, prec)
    assert d <= 0


@pytest.mark.parametrize("prec", ["ref32", "ref64"])
def test_collision_kat(prec):
    assert O.prim_collision([0.5, 0.5, 1.05], [0.6, 0.5, 1.05], 0.1, BOX, prec) == 1
    assert O.prim_collision([0.5, 0.5, 1.2], [0.6, 0.5, 1.2], 0.1, BOX, prec) == 0
    assert O.prim_collision([-1, 0.5, 0.5], [2, 0.5, 0.5], 0.0, BOX, prec) == 1
    assert O.prim_collision([3, 3, 3], [4, 4, 4], 0.5, BOX, prec) == 0


def test_translation_invariance():
    rng = np.random.default_rng(1)
    shift = np.float32(0.5)
    for _ in range(500):
        a, b = rng.uniform(-1, 2, 3).astype(np.float32), rng.uniform(-1, 2, 3).astype(np.float32)
        d0 = O.prim_distance(a, b, 0.05, BOX, "ref64")[0]
        d1 = O.prim_distance(a + shift, b + shift, 0.05, BOX + shift, "ref64")[0]
        assert abs(d0 - d1) < 1e-6


def test_parallel_and_degenerate_segments():
    lib = O.lib()
    import ctypes
    fp = ctypes.POINTER(ctypes.c_float)
    P = lambda x: np.ascontiguousarray(x, np.float32).ctypes.data_as(fp)
    # parallel segments 0.3 apart, overlapping in projection
    d = lib.orc_prim_segseg(P([0, 0, 0]), P([1, 0, 0]), P([0.2, 0.3, 0]), P([0.8, 0.3, 0]), 64, None)
    assert abs(d - float(np.float32(0.3))) < 1e-12
    # parallel, disjoint in projection: endpoint distance
    d = lib.orc_prim_segseg(P([0, 0, 0]), P([1, 0, 0]), P([2, 0.3, 0]), P([3, 0.3, 0]), 64, None)
    assert abs(d - math.hypot(1.0, 0.3)) < 1e-7
    # crossing segments: below EQUALITY_THRESHOLD -> exactly 0
    d = lib.orc_prim_segseg(P([0, 0, 0]), P([1, 1, 0]), P([0, 1, 0]), P([1, 0, 0]), 64, None)
    assert d == 0.0


def test_min_dist_tol_and_ground_rule():
    rb = robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    g_aabb, g_tol = scenes.ground_box()
    scene = scenes.Scene(g_aabb[None, :], np.array([g_tol]), np.array([1], np.uint8))
    q = np.zeros((1, 6), np.float32)
    q[0, 1] = -0.3   # lean back: links stay well above the ground
    v, d, p = O.check_configs(rb, scene, q, prec="ref64")
    # every ground distance beyond min_dist_tol (0.05) becomes MAX_DISTANCE
    assert v[0] == 1 and d[0] == 1000.0 and np.all(p[0] == 1000.0)
    # links below ground_included never see the ground even when they would touch it
    rb.set_ground_included(6)
    q2 = np.zeros((1, 6), np.float32)
    v2, d2, _ = O.check_configs(rb, scene, q2, prec="ref64")
    assert v2[0] == 1 and d2[0] == 1000.0


def test_early_exit_profile_shape():
    rb = robots.planar_2dof(radius=0.0)
    # box crossed by link 1 only (link 0 spans x in [0, 1])
    scene = scenes.Scene(np.array([[1.5, -0.1, -0.1, 1.6, 0.1, 0.1], [5, 5, -0.1, 6, 6, 0.1]], np.float32))
    v, d, p = O.check_configs(rb, scene, np.zeros((1, 2), np.float32), prec="ref64")
    assert v[0] == 0 and d[0] == 0.0
    # link 0: full minimum over both boxes; link 1: the hit value (<= 0)
    assert abs(p[0, 0] - 0.5) < 1e-6 and p[0, 1] <= 0
    # a 3-link chain colliding at link 0 has zeros after the hit
    rb3 = robots.spatial(10, radius=0.03)
    scene3 = scenes.Scene(np.array([[-0.05, -0.05, 0.02, 0.05, 0.05, 0.08]], np.float32))
    v, d, p = O.check_configs(rb3, scene3, np.zeros((1, 10), np.float32), prec="ref64")
    assert v[0] == 0 and p[0, 0] <= 0 and np.all(p[0, 1:] == 0)


def test_sincos_accuracy():
    x = np.linspace(-8, 8, 200001)
    s, c = O.sincos(x)
    ulp = lambda v: np.spacing(np.abs(v)) + 1e-300
    assert (np.abs(s - np.sin(x)) / ulp(np.sin(x))).max() <= 1.0
    assert (np.abs(c - np.cos(x)) / ulp(np.cos(x))).max() <= 1.0


def test_box_aabb_rule_matches_host_generator():
    rng = np.random.default_rng(3)
    for _ in range(200):
        dim, pos = rng.uniform(0.01, 1, 3), rng.uniform(-2, 2, 3)
        for quat in ([0, 0, 0, 1], rng.normal(size=4) / 2):
            assert np.array_equal(O.box_aabb(dim, pos, quat), scenes.box_aabb(dim, pos, quat))
    # rotated boxes become the cube pos +- |dim/2|
    a = scenes.box_aabb([0.2, 0.4, 0.4], [0, 0, 0], [0.1, 0.2, 0.3, 0.9])
    assert np.allclose(a, [-0.3, -0.3, -0.3, 0.3, 0.3, 0.3])
