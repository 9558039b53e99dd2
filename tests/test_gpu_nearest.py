"""GPU parity of computeDistance with nearest points (RealVectorSpace.cpp:318-392)
and computeDistanceUnderestimation (:402-446) against the oracle.

Bars: fp32_ref bit-equal to ref32 (the reference's own numerics); fp64
bit-equal to ref64 (its points rounded to float).  Nearest points are compared
where the reference has them (nearest_valid = 1); elsewhere the reference
returns nullptr and only the flag is compared.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

pytestmark = pytest.mark.gpu

FORMS = [("fp64", "ref64"), ("fp32_ref", "ref32")]


def _near_gpu(engine, sid, q, L, n, prec):
    C = q.shape[0]
    qd = torch.from_numpy(q).cuda()
    d = torch.zeros(C, dtype=torch.float64, device="cuda")
    p = torch.zeros((C, L), dtype=torch.float32, device="cuda")
    near = torch.zeros((C, n, 6, L), dtype=torch.float32, device="cuda")
    nv = torch.zeros(C, dtype=torch.uint8, device="cuda")
    engine.distance_nearest(sid, qd, d, p, near, nv, prec)
    engine.sync()
    return d.cpu().numpy(), p.cpu().numpy(), near.cpu().numpy(), nv.cpu().numpy()


def _under_gpu(engine, sid, q, near, L, prec):
    C = q.shape[0]
    d = torch.zeros(C, dtype=torch.float64, device="cuda")
    p = torch.zeros((C, L), dtype=torch.float32, device="cuda")
    comp = torch.zeros(C, dtype=torch.uint8, device="cuda")
    engine.distance_underestimation(sid, torch.from_numpy(q).cuda(), torch.from_numpy(near).cuda(), d, p, comp, prec)
    engine.sync()
    return d.cpu().numpy(), p.cpu().numpy(), comp.cpu().numpy()


def _check(robot, scene, q, engine, prec, oprec):
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    L, n = robot.num_links, scene.n
    d, p, near, nv = _near_gpu(engine, sid, q, L, n, prec)
    rd, rp, rnear, rnv = O.distance_nearest(robot, scene, q, prec=oprec)
    assert np.array_equal(nv, rnv)
    assert np.array_equal(d.view(np.uint64), rd.view(np.uint64))
    assert np.array_equal(p.view(np.uint32), rp.view(np.uint32))
    sel = nv == 1
    assert np.array_equal(near[sel].view(np.uint32), rnear[sel].view(np.uint32))
    # underestimation from the GPU's own nearest points and from the oracle's
    for src in (near, rnear):
        src = src.copy()
        src[~sel] = 0.0
        ud, up, uc = _under_gpu(engine, sid, q, src, L, prec)
        rud, rup, ruc = O.distance_underestimation(robot, n, q, src, prec=oprec)
        assert np.array_equal(uc, ruc)
        assert np.array_equal(ud.view(np.uint64), rud.view(np.uint64))
        full = uc == 1
        assert np.array_equal(up[full].view(np.uint32), rup[full].view(np.uint32))
    engine.destroy_scene(sid)
    return nv


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_nearest_xarm6_with_ground(engine, prec, oprec):
    """xArm6 with the ground skipped for its first links: the skipped pairs carry
    the reference's (0, 0, 0), (0, 0, -MAX_DISTANCE) marker."""
    robot, scene, q = scenes.xarm6_workload(2048, seed=61)
    nv = _check(robot, scene, q, engine, prec, oprec)
    assert 0 < nv.sum() < len(nv)   # both outcomes occur


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_nearest_spatial_sparse(engine, prec, oprec):
    """A 14-DOF chain among small boxes: most configurations are free, so the
    nearest points and the underestimation are exercised on every region of
    the capsule-box tree."""
    robot = robots.spatial(14, radius=0.03)
    rng = np.random.default_rng(62)
    boxes = [scenes.box_aabb(rng.uniform(0.01, 0.05, 3), c)
             for c in scenes._ball(rng, 120, scenes.SPATIAL_WS_CENTER, 2.0)]
    scene = scenes.Scene(np.array(boxes), tol=rng.uniform(0.05, 1.5, 120).astype(np.float32))
    q = scenes.uniform_configs(rng, 1024, 14)
    nv = _check(robot, scene, q, engine, prec, oprec)
    assert nv.sum() > 100


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_nearest_planar(engine, prec, oprec):
    robot, scene, q = scenes.planar_2dof_workload(4096, seed=63)
    _check(robot, scene, q, engine, prec, oprec)


def test_nearest_empty_scene(engine):
    robot = robots.spatial(10, radius=0.03)
    scene = scenes.Scene(np.zeros((0, 6), np.float32))
    q = scenes.uniform_configs(np.random.default_rng(64), 33, 10)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    d, p, near, nv = _near_gpu(engine, sid, q, robot.num_links, 0, "fp64")
    assert np.all(nv == 1) and np.all(d == 1000.0) and np.all(p == 1000.0)
    engine.destroy_scene(sid)
