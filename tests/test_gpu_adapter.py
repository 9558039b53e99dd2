"""The C++ RealVectorSpaceGPU adapter, driven like a planner drives
base::RealVectorSpace (tests/adapter_driver.cpp), against the oracle:
isValid(q), isValid(q1, q2), computeDistance with its cache, nearest points
and skeleton write-back, computeDistanceUnderestimation, and the batched forms.
In RPM_PREC_FP32_REF every output is bit-equal to the reference's numerics."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from rpmplv2_gb300 import _abi, build, robots, scenes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    exe = os.path.join(build.OUT_DIR, "adapter_driver")
    cmd = [build.nvcc(), "-std=c++17", "-O2", "-x", "c++", os.path.join(HERE, "adapter_driver.cpp"),
           *build.adapter_flags(), "-L", build.OUT_DIR, "-lrpm_adapter", "-lrpm_gb300",
           "-Xlinker", "-rpath=" + build.OUT_DIR, "-lcudart", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def _run(exe, robot, scene, q, q1, q2, prec):
    C, D, E, n = q.shape[0], robot.num_dofs, q1.shape[0], scene.n
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(np.array([prec, C, E, n, D], np.int32).tobytes())
            f.write(bytes(robot.desc))
            f.write(scene.aabb.tobytes()); f.write(scene.tol.tobytes()); f.write(scene.flags.tobytes())
            f.write(q.tobytes()); f.write(q1.tobytes()); f.write(q2.tobytes())
        subprocess.run([exe, fin, fout], check=True)
        raw = open(fout, "rb").read()
    out, off = {}, 0
    NS = n * 6 * D
    for name, dt, cnt in (("valid", np.uint8, C), ("valid_b", np.uint8, C), ("dist", np.float32, C),
                          ("prof", np.float32, C * D), ("has_near", np.uint8, C), ("near", np.float32, C * NS),
                          ("cached_ok", np.uint8, C), ("skel", np.float32, C * 3 * (D + 1)), ("under", np.float32, C),
                          ("under_set", np.uint8, C), ("under_prof", np.float32, C * D), ("dist_b", np.float32, C),
                          ("edge", np.uint8, E), ("edge_b", np.uint8, E)):
        nb = np.dtype(dt).itemsize * cnt
        out[name] = np.frombuffer(raw[off:off + nb], dt).copy()
        off += nb
    assert off == len(raw)
    out["prof"] = out["prof"].reshape(C, D)
    out["near"] = out["near"].reshape(C, n, 6, D)
    out["skel"] = out["skel"].reshape(C, D + 1, 3)
    out["under_prof"] = out["under_prof"].reshape(C, D)
    return out


def _bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.parametrize("workload", ["xarm6", "spatial14"])
def test_adapter_reference_numerics(driver, workload):
    rng = np.random.default_rng(71)
    if workload == "xarm6":
        robot, scene, q = scenes.xarm6_workload(96, seed=72)
    else:
        robot = robots.spatial(14, radius=0.03)
        boxes = [scenes.box_aabb(rng.uniform(0.01, 0.06, 3), c) for c in scenes._ball(rng, 80, scenes.SPATIAL_WS_CENTER, 2.0)]
        scene = scenes.Scene(np.array(boxes))
        q = scenes.uniform_configs(rng, 96, 14)
    D = robot.num_dofs
    q1 = scenes.uniform_configs(rng, 64, D)
    q2 = (q1 + rng.uniform(-0.4, 0.4, q1.shape)).astype(np.float32)
    out = _run(driver, robot, scene, q, q1, q2, _abi.RPM_PREC_FP32_REF)
    rv, rd, rp = O.check_configs(robot, scene, q, prec="ref32")
    assert np.array_equal(out["valid"], rv) and np.array_equal(out["valid_b"], rv)
    nd, npf, nnear, nnv = O.distance_nearest(robot, scene, q, prec="ref32")
    assert _bits(out["dist"], nd.astype(np.float32)) and _bits(out["prof"], npf)
    assert np.array_equal(out["has_near"], nnv)
    sel = nnv == 1
    assert _bits(out["near"][sel], nnear[sel])
    assert out["cached_ok"].all()
    assert _bits(out["skel"], O.skeleton(robot, q, prec="ref32").astype(np.float32))
    assert _bits(out["dist_b"], rd.astype(np.float32))
    # underestimation at configuration c+1 from the nearest points of c
    qn = np.roll(q, -1, axis=0)
    ud, up, uc = O.distance_underestimation(robot, scene.n, qn, nnear, prec="ref32")
    assert np.array_equal(out["under_set"][sel], uc[sel])
    assert _bits(out["under"][sel], np.where(uc[sel] == 1, ud[sel], 0.0).astype(np.float32))
    done = sel & (uc == 1)
    assert _bits(out["under_prof"][done], up[done])
    ev, ek = O.check_edges(robot, scene, q1, q2, step=0.0, num_checks=10, prec="ref32")
    assert np.array_equal(out["edge"], ev) and np.array_equal(out["edge_b"], ev)
    assert 0 < sel.sum() < len(sel) or workload == "spatial14"


def test_adapter_fp32_recheck_booleans(driver):
    """The default form (FP32 + FP64 recheck): booleans equal to ref64."""
    robot, scene, q = scenes.xarm6_workload(128, seed=73)
    rng = np.random.default_rng(74)
    q1 = scenes.uniform_configs(rng, 64, 6)
    q2 = (q1 + rng.uniform(-0.4, 0.4, q1.shape)).astype(np.float32)
    out = _run(driver, robot, scene, q, q1, q2, _abi.RPM_PREC_FP32_RECHECK)
    rv, rd, rp = O.check_configs(robot, scene, q, prec="ref64")
    assert np.array_equal(out["valid"], rv) and np.array_equal(out["valid_b"], rv)
    assert np.abs(out["dist_b"].astype(np.float64) - rd).max() <= 1e-5
    # the single-state computeDistance runs the FP64 form: its distance rounded to float
    nd, npf, nnear, nnv = O.distance_nearest(robot, scene, q, prec="ref64")
    assert _bits(out["dist"], nd.astype(np.float32)) and _bits(out["prof"], npf)
    assert np.array_equal(out["has_near"], nnv)
    sel = nnv == 1
    assert _bits(out["near"][sel], nnear[sel])
    ev, _ = O.check_edges(robot, scene, q1, q2, step=0.0, num_checks=10, prec="ref64")
    assert np.array_equal(out["edge"], ev) and np.array_equal(out["edge_b"], ev)


@pytest.fixture(scope="module")
def env_driver():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build.build()
    exe = os.path.join(build.OUT_DIR, "adapter_env_driver")
    cmd = [build.nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-x", "c++",
           os.path.join(HERE, "adapter_env_driver.cpp"), *build.adapter_flags(), "-L", build.OUT_DIR,
           "-lrpm_adapter", "-lrpm_gb300", "-Xlinker", "-rpath=" + build.OUT_DIR, "-lcudart", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def _quat(rng):
    u = rng.normal(size=4)
    return (u / np.linalg.norm(u)).astype(np.float32)


@pytest.mark.parametrize("prec", [_abi.RPM_PREC_FP32_REF, _abi.RPM_PREC_FP32_RECHECK])
def test_adapter_follows_the_environment(env_driver, prec):
    """The reference's constructor RealVectorSpaceGPU(D, robot, env): the space
    keeps ss->robot and ss->env, describes the robot by its type, reads the
    obstacles as fcl world AABBs with their labels and tolerances, and follows
    the environment as MotionValidity::check moves it in place
    (env->updateEnvironment(dt), then ss->isValid(q) and computeDistance);
    removing and adding an object rebuilds the scene.  Every step's results
    equal the oracle on the AABBs the environment held at that step."""
    rng = np.random.default_rng(91)
    D, S, K, dt = 6, 6, 64, 0.05
    robot = robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    recs = [[1.5, 1.5, 0.1, 0, 0, -0.05, 0, 0, 0, 1, 1, 0.05]]   # the ground (label, min_dist_tol 0.05)
    for j in range(36):
        c = np.array([0, 0, 0.267]) + rng.uniform(-0.8, 0.8, 3)
        dim = rng.uniform(0.04, 0.12, 3)
        quat = _quat(rng) if j % 6 == 0 else np.array([0, 0, 0, 1], np.float32)
        code, last = (2, rng.uniform(0.5, 1.6)) if j % 7 == 0 else (0, 0.0)
        recs.append([*dim, *c, *quat, code, last])
    boxes = np.array(recs, np.float32)
    extra = np.array([0.1, 0.1, 0.1, 0.3, -0.3, 0.5, 0, 0, 0, 1, 0, 0], np.float32)
    q = scenes.uniform_configs(rng, (S + 1) * K, D)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(np.array([prec, S, K, len(boxes), D, 2], np.int32).tobytes())
            f.write(b"xarm6".ljust(32, b"\0"))
            f.write(robot.capsule_radius.tobytes())
            f.write(np.array([0.1, dt], np.float32).tobytes())
            f.write(boxes.tobytes()); f.write(extra.tobytes()); f.write(q.tobytes())
        subprocess.run([env_driver, fin, fout], check=True)
        raw = open(fout, "rb").read()
    code = boxes[:, 10].astype(int)
    tol = np.where(code == 1, boxes[:, 11], 1000.0).astype(np.float32)
    flags = np.where(code == 1, _abi.RPM_OBS_GROUND, np.where(code == 2, _abi.RPM_OBS_DYNAMIC, 0)).astype(np.uint8)
    off, moved = 0, 0
    prev = None
    oracle = "ref32" if prec == _abi.RPM_PREC_FP32_REF else "ref64"
    for s in range(S + 2):
        cnt = int(np.frombuffer(raw[off:off + 4], np.int32)[0]); off += 4
        aabb = np.frombuffer(raw[off:off + 24 * cnt], np.float32).reshape(cnt, 6).copy(); off += 24 * cnt
        res = np.frombuffer(raw[off:off + 5 * K], np.uint8).reshape(K, 5); off += 5 * K
        v = res[:, 0].copy()
        dist = res[:, 1:].copy().view(np.float32).reshape(K)
        if s == S + 1:   # object 0 removed, one static box added
            tol = np.concatenate([tol[1:], [1000.0]]).astype(np.float32)
            flags = np.concatenate([flags[1:], [0]]).astype(np.uint8)
        elif prev is not None:
            moved += int((aabb != prev).any(axis=1).sum())
        prev = aabb
        scene = scenes.Scene(aabb, tol, flags)
        row = min(s, S)
        qs = q[row * K:(row + 1) * K]
        rv, rd, _ = O.check_configs(robot, scene, qs, prec=oracle, want=("valid", "dist"))
        assert np.array_equal(v, rv), "step %d" % s
        nd, _, _, _ = O.distance_nearest(robot, scene, qs, prec=oracle)
        assert _bits(dist, nd.astype(np.float32)), "step %d" % s
    assert off == len(raw)
    assert moved >= S * 5   # the dynamic boxes moved every step
