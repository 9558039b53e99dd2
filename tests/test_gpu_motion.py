"""GPU parity of MotionValidity::check with moving boxes (rpm_motion_validity)
against the oracle: bit-equal validity and check counts in the reference's
float numerics and in FP64."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import _abi, scenes, serve
from test_oracle_motion import movers_of

pytestmark = pytest.mark.gpu


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name,n", [("xarm6", 40), ("spatial_10dof", 200), ("planar_2dof", 8)])
def test_motion_validity(engine, name, n):
    rng = np.random.default_rng(92)
    rb = serve.make_robot(name)
    scene = serve._scene_for(rb, rng, n)
    D = rb.num_dofs
    # five boxes, one of them rotated, sweeping -x fast enough to cross the workspace
    first = 1 if name == "xarm6" else 0
    idx = rng.choice(np.arange(first, scene.n), size=5, replace=False)
    specs, quats = [], []
    for k, j in enumerate(idx):
        dim = rng.uniform(0.05, 0.3, 3).astype(np.float32)
        pos = rng.uniform(-1.0, 1.0, 3).astype(np.float32)
        pos[0] += 1.5
        quat = (0.0, 0.0, 0.0, 1.0) if k else tuple(np.array([0.1, 0.2, 0.3, 0.9]) / np.linalg.norm([0.1, 0.2, 0.3, 0.9]))
        scene.aabb[j] = scenes.box_aabb(dim, pos, quat)
        scene.flags[j] |= _abi.RPM_OBS_DYNAMIC
        specs.append((int(j), float(rng.uniform(10.0, 60.0)), dim, pos))
        quats.append(quat)
    mv = movers_of(specs, quats)
    M = 1500
    q1 = scenes.uniform_configs(rng, M, D)
    q2 = (q1 + rng.uniform(-0.6, 0.6, q1.shape)).astype(np.float32)
    q2[:20] = q1[:20]                                   # standing still while the boxes move
    sid = engine.create_scene(engine.upload_robot(rb), scene)
    for prec, oprec in (("fp32_ref", "ref32"), ("fp64", "ref64")):
        v = torch.zeros(M, dtype=torch.uint8, device="cuda")
        k = torch.zeros(M, dtype=torch.int32, device="cuda")
        engine.motion_validity(sid, _t(q1), _t(q2), mv, 0.05, 12, v, k, precision=prec)
        engine.sync()
        rv, rk = O.motion_validity(rb, scene, q1, q2, mv, 0.05, 12, prec=oprec)
        assert np.array_equal(v.cpu().numpy(), rv)
        assert np.array_equal(k.cpu().numpy(), rk)
    # the moving boxes matter: the same motions against the boxes held still differ
    still = movers_of([(j, 0.0, d, p) for (j, _, d, p) in specs], quats)
    sv, _ = O.motion_validity(rb, scene, q1, q2, still, 0.05, 12)
    assert not np.array_equal(sv, rv)
    if name != "planar_2dof":   # the 1 m planar links meet the sweeping boxes on every motion
        assert 0 < rv.sum() < M
    engine.destroy_scene(sid)


def test_move_straight_updates_the_scene(engine):
    """MotionValidity::check moves the environment once per check it makes; moving the
    device scene by those steps leaves it equal to the oracle's moved scene."""
    rng = np.random.default_rng(93)
    rb = serve.make_robot("spatial_10dof")
    scene = serve._scene_for(rb, rng, 60)
    specs = []
    for j in range(3):
        dim = rng.uniform(0.05, 0.2, 3).astype(np.float32)
        pos = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        scene.aabb[j] = scenes.box_aabb(dim, pos)
        scene.flags[j] |= _abi.RPM_OBS_DYNAMIC
        specs.append((j, float(rng.uniform(5.0, 20.0)), dim, pos))
    mv = movers_of(specs)
    sid = engine.create_scene(engine.upload_robot(rb), scene)
    q1 = scenes.uniform_configs(rng, 1, 10)
    q2 = (q1 + 0.3).astype(np.float32)
    N, T = 10, 0.05
    k = torch.zeros(1, dtype=torch.int32, device="cuda")
    v = torch.zeros(1, dtype=torch.uint8, device="cuda")
    engine.motion_validity(sid, _t(q1), _t(q2), mv, T, N, v, k)
    engine.sync()
    steps = int(k.cpu().numpy()[0])
    engine.move_straight(sid, mv, np.float32(T) / np.float32(N), steps)
    # the oracle's view of the same motion of the boxes
    dt = np.float32(np.float32(T) / np.float32(N))
    moved = scenes.Scene(scene.aabb.copy(), scene.tol.copy(), scene.flags.copy())
    for (j, vel, dim, pos), box in zip(specs, mv):
        p = pos.copy()
        for _ in range(steps):
            p[0] = np.float32(p[0] - np.float32(dt * np.float32(vel)))
        assert np.array_equal(np.array(box.pos[:], np.float32), p)
        moved.aabb[j] = scenes.box_aabb(dim, p)
    q = scenes.uniform_configs(rng, 2048, 10)
    vd = torch.zeros(2048, dtype=torch.uint8, device="cuda")
    dd = torch.zeros(2048, dtype=torch.float64, device="cuda")
    engine.check_configs(sid, _t(q), "fp32_ref", vd, dd, None)
    engine.sync()
    rv, rd, _ = O.check_configs(rb, moved, q, prec="ref32", want=("valid", "dist"))
    assert np.array_equal(vd.cpu().numpy(), rv) and np.array_equal(dd.cpu().numpy().view(np.uint64), rd.view(np.uint64))
    engine.destroy_scene(sid)
