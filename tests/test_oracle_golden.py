"""The oracle against the committed golden fixtures (tests/golden/golden.npz,
made by tests/golden/make_golden.py) and against the reference's own
CollisionAndDistance.cpp where its tree is present."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("prec", ["ref32", "ref64"])
def test_planar(prec):
    robot = robots.planar_2dof(radius=0.0)
    scene = scenes.Scene(G["planar_aabb"])
    v, d, p = O.check_configs(robot, scene, G["planar_q"], prec=prec)
    assert bits_equal(v, G["planar_%s_valid" % prec])
    assert bits_equal(d, G["planar_%s_dist" % prec])
    assert bits_equal(p, G["planar_%s_prof" % prec])


@pytest.mark.parametrize("prec", ["ref32", "ref64"])
def test_xarm6(prec):
    robot = robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    scene = scenes.Scene(G["xarm6_aabb"], G["xarm6_tol"], G["xarm6_flags"])
    v, d, p = O.check_configs(robot, scene, G["xarm6_q"], prec=prec)
    assert bits_equal(v, G["xarm6_%s_valid" % prec])
    assert bits_equal(d, G["xarm6_%s_dist" % prec])
    assert bits_equal(p, G["xarm6_%s_prof" % prec])
    assert bits_equal(O.skeleton(robot, G["xarm6_q"][:64], prec="ref64"), G["xarm6_skel64"])
    assert bits_equal(O.skeleton(robot, G["xarm6_q"][:64], prec="ref32"), G["xarm6_skel32"])


@pytest.mark.parametrize("prec", ["ref32", "ref64"])
def test_edges(prec):
    robot = robots.spatial(10, radius=0.03)
    scene = scenes.Scene(G["edges_aabb"])
    v, k = O.check_edges(robot, scene, G["edges_q1"], G["edges_q2"], step=np.float32(0.05), prec=prec)
    assert bits_equal(v, G["edges_%s_valid" % prec])
    assert bits_equal(k, G["edges_%s_checks" % prec])
    assert 1 <= k.min() and k.max() <= 40


def test_mixed_dof():
    scene = scenes.Scene(G["mixed_aabb"])
    for dofs in (14, 18, 22):
        robot = robots.spatial(dofs, radius=0.03)
        v, d, p = O.check_configs(robot, scene, G["mixed%d_q" % dofs], prec="ref64")
        assert bits_equal(v, G["mixed%d_ref64_valid" % dofs])
        assert bits_equal(d, G["mixed%d_ref64_dist" % dofs])
        assert bits_equal(p, G["mixed%d_ref64_prof" % dofs])


def test_primitives_against_fixture():
    A, B, obs, r = G["prim_A"], G["prim_B"], G["prim_obs"], G["prim_r"]
    coll = np.array([O.prim_collision(A[i], B[i], r[i], obs[i], "ref32") for i in range(len(r))], np.uint8)
    dist = np.array([O.prim_distance(A[i], B[i], r[i], obs[i], "ref32")[0] for i in range(len(r))], np.float32)
    assert bits_equal(coll, G["prim_ref32_coll"])
    assert bits_equal(dist, G["prim_ref32_dist"])
    if "prim_reference_coll" in G:
        # answered by the reference's own source when the fixture was made
        assert bits_equal(coll, G["prim_reference_coll"])
        assert bits_equal(dist, G["prim_reference_dist"])


def test_primitives_against_reference_source():
    R = O.ref()
    if R is None:
        pytest.skip("reference tree not present")
    import ctypes
    fp = ctypes.POINTER(ctypes.c_float)
    rng = np.random.default_rng(5)
    for it in range(20000):
        c = rng.uniform(-0.3, 0.3, 3).astype(np.float32)
        h = rng.uniform(0.01, 0.2, 3).astype(np.float32)
        o = np.concatenate([c - h, c + h]).astype(np.float32)
        a = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        b = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        if it % 5 == 0:
            b[it % 3] = a[it % 3]
        r = float(rng.choice([0.0, 0.03, 0.1]))
        P = lambda x: np.ascontiguousarray(x).ctypes.data_as(fp)
        assert R.ref_collision(P(a), P(b), r, P(o)) == O.prim_collision(a, b, r, o, "ref32")
        rpts = np.zeros(6, np.float32)
        rhas = ctypes.c_int()
        rd = np.float32(R.ref_distance(P(a), P(b), r, P(o), P(rpts), ctypes.byref(rhas)))
        od, opts, ohas = O.prim_distance(a, b, r, o, "ref32")
        assert rd.tobytes() == np.float32(od).tobytes()
        # the nearest points (robot point, obstacle point) of CapsuleToBox, or none
        assert bool(rhas.value) == ohas
        if ohas:
            assert rpts.tobytes() == opts.tobytes(), (it, rpts, opts)


def test_adversarial_primitives_against_fixture():
    """The directed edge cases (parallel, degenerate, on-plane, snap-distance):
    the oracle reproduces its committed answers in both numerics, and its FP32
    restatement equals the reference's own source wherever that source is
    defined (adv_undefined marks its uninitialised-matrix reads)."""
    import ctypes
    A, B, X, r, kind = (G[k] for k in ("adv_A", "adv_B", "adv_X", "adv_r", "adv_kind"))
    fp = ctypes.POINTER(ctypes.c_float)
    P = lambda a: np.ascontiguousarray(a).ctypes.data_as(fp)
    L = O.lib()
    n = len(r)
    v32, v64, und = np.zeros(n), np.zeros(n), np.zeros(n, np.uint8)
    O.undefined_hits()
    for i in range(n):
        if kind[i] == 0:
            v32[i] = O.prim_collision(A[i], B[i], r[i], X[i], "ref32")
            v64[i] = O.prim_collision(A[i], B[i], r[i], X[i], "ref64")
        elif kind[i] == 1:
            v32[i] = O.prim_distance(A[i], B[i], r[i], X[i], "ref32")[0]
            v64[i] = O.prim_distance(A[i], B[i], r[i], X[i], "ref64")[0]
            und[i] = 1 if O.undefined_hits() else 0
        else:
            v32[i] = L.orc_prim_segseg(P(A[i]), P(B[i]), P(X[i][:3]), P(X[i][3:]), 32, None)
            v64[i] = L.orc_prim_segseg(P(A[i]), P(B[i]), P(X[i][:3]), P(X[i][3:]), 64, None)
    nan_eq = lambda a, b: np.all((np.isnan(a) & np.isnan(b)) | (a == b))
    assert nan_eq(v32, G["adv_ref32"]) and nan_eq(v64, G["adv_ref64"])
    assert np.array_equal(und, G["adv_undefined"])
    if "adv_reference" in G:
        d = und == 0
        assert nan_eq(v32[d].astype(np.float32), G["adv_reference"][d].astype(np.float32))
