"""GPU parity of the mixed-DOF batch launch, the edge checks and the golden
fixtures.  Bars as in test_gpu_parity: exact forms bit-equal to the oracle,
FP32+recheck with 0 isValid flips and distances within 1e-5 m."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

pytestmark = pytest.mark.gpu
G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def _t(a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda() if dtype is None else torch.zeros(a, dtype=dtype, device="cuda")


@pytest.mark.parametrize("prec,oracle_prec", [("fp64", "ref64"), ("fp32_ref", "ref32"), ("fp32_recheck", "ref64")])
def test_mixed_dof_single_launch(engine, prec, oracle_prec):
    scene, parts = scenes.mixed_dof_workload(counts=(2048, 3072, 3072), seed=31)
    items, outs = [], []
    for robot, q in parts:
        sid = engine.create_scene(engine.upload_robot(robot), scene)
        C, L = q.shape[0], robot.num_links
        v, d, p = _t(C, torch.uint8), _t(C, torch.float64), torch.zeros((C, L), device="cuda")
        items.append((sid, _t(q), v, d, p))
        outs.append((robot, q, v, d, p))
    engine.check_batch(items, prec)
    engine.sync()
    for robot, q, v, d, p in outs:
        rv, rd, rp = O.check_configs(robot, scene, q, prec=oracle_prec)
        v, d, p = v.cpu().numpy(), d.cpu().numpy(), p.cpu().numpy()
        assert np.array_equal(v, rv)
        if prec == "fp32_recheck":
            assert np.abs(d - rd).max() <= 1e-5 and np.abs(p - rp).max() <= 1e-5
        else:
            assert np.array_equal(d.view(np.uint64), rd.view(np.uint64))
            assert np.array_equal(p.view(np.uint32), rp.view(np.uint32))
    for it in items:
        engine.destroy_scene(it[0])


def test_recheck_groups_of_many_segments(engine):
    """FP32 + recheck over 20 requests that each want isValid and a distance:
    40 launch segments, so the launches form two recheck groups (at most 32
    segments each) that share the recheck lists in turn.  0 flips against
    ref64, distances within 1e-5 m."""
    robot, scene, q = scenes.xarm6_workload(20 * 512, seed=41)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    items = []
    for k in range(20):
        items.append((sid, _t(q[k * 512:(k + 1) * 512]), _t(512, torch.uint8), _t(512, torch.float64), None))
    engine.check_batch(items, "fp32_recheck")
    engine.sync()
    rv, rd, _ = O.check_configs(robot, scene, q, prec="ref64")
    v = np.concatenate([it[2].cpu().numpy() for it in items])
    d = np.concatenate([it[3].cpu().numpy() for it in items])
    assert np.array_equal(v, rv)
    assert np.abs(d - rd).max() <= 1e-5
    engine.destroy_scene(sid)


@pytest.mark.parametrize("prec,oracle_prec", [("fp64", "ref64"), ("fp32_ref", "ref32"), ("fp32_recheck", "ref64")])
def test_edges_uneven(engine, prec, oracle_prec):
    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(6000, seed=32)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    v, k = _t(q1.shape[0], torch.uint8), _t(q1.shape[0], torch.int32)
    engine.check_edges(sid, _t(q1), _t(q2), v, k, step=float(step), precision=prec)
    engine.sync()
    rv, rk = O.check_edges(robot, scene, q1, q2, step=step, prec=oracle_prec)
    assert np.array_equal(v.cpu().numpy(), rv)
    assert np.array_equal(k.cpu().numpy(), rk)
    engine.destroy_scene(sid)


def test_edges_fixed_count_graphs_and_autotune(engine):
    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(3000, seed=33)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    q1d, q2d = _t(q1), _t(q2)
    v = _t(q1.shape[0], torch.uint8)
    rv, rk = O.check_edges(robot, scene, q1, q2, step=0.0, num_checks=10, prec="ref64")
    engine.set_graphs(True)
    for _ in range(2):   # capture, then replay
        v.fill_(7)
        engine.check_edges(sid, q1d, q2d, v, None, step=0.0, num_checks=10, precision="fp32_recheck")
        engine.sync()
        assert np.array_equal(v.cpu().numpy(), rv)
    engine.set_graphs(False)
    best = engine.autotune_edges(sid, q1d, q2d, v, step=float(step), precision="fp32_recheck")
    assert best["layout"] in ("lane", "warp") and best["ms"] > 0
    if best["layout"] == "lane":
        assert best["ctas_per_sm"] in (1, 2, 3, 4, 6, 8)
    v.fill_(7)
    engine.check_edges(sid, q1d, q2d, v, None, step=float(step), precision="fp32_recheck")
    engine.sync()
    rv2, _ = O.check_edges(robot, scene, q1, q2, step=step, prec="ref64")
    assert np.array_equal(v.cpu().numpy(), rv2)
    engine.destroy_scene(sid)


@pytest.mark.parametrize("prec,tag", [("fp64", "ref64"), ("fp32_ref", "ref32")])
def test_golden_fixtures_on_gpu(engine, prec, tag):
    cases = [(robots.planar_2dof(radius=0.0), scenes.Scene(G["planar_aabb"]), G["planar_q"], "planar"),
             (robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2),
              scenes.Scene(G["xarm6_aabb"], G["xarm6_tol"], G["xarm6_flags"]), G["xarm6_q"], "xarm6")]
    for robot, scene, q, name in cases:
        sid = engine.create_scene(engine.upload_robot(robot), scene)
        C, L = q.shape[0], robot.num_links
        v, d, p = _t(C, torch.uint8), _t(C, torch.float64), torch.zeros((C, L), device="cuda")
        engine.check_configs(sid, _t(q), prec, v, d, p)
        engine.sync()
        assert np.array_equal(v.cpu().numpy(), G["%s_%s_valid" % (name, tag)])
        assert np.array_equal(d.cpu().numpy().view(np.uint64), G["%s_%s_dist" % (name, tag)].view(np.uint64))
        assert np.array_equal(p.cpu().numpy().view(np.uint32), G["%s_%s_prof" % (name, tag)].view(np.uint32))
        engine.destroy_scene(sid)
    robot = robots.spatial(10, radius=0.03)
    sid = engine.create_scene(engine.upload_robot(robot), scenes.Scene(G["edges_aabb"]))
    v, k = _t(512, torch.uint8), _t(512, torch.int32)
    engine.check_edges(sid, _t(G["edges_q1"]), _t(G["edges_q2"]), v, k, step=0.05, precision=prec)
    engine.sync()
    assert np.array_equal(v.cpu().numpy(), G["edges_%s_valid" % tag])
    assert np.array_equal(k.cpu().numpy(), G["edges_%s_checks" % tag])
    engine.destroy_scene(sid)


def _edge_items(engine, rng):
    """Edge sets of several robots and scene sizes (both layouts), uneven and fixed discretisations."""
    from rpmplv2_gb300 import serve
    specs = [("planar_2dof", 8, 300, 0.05), ("xarm6", 40, 700, 0.05), ("spatial_10dof", 250, 900, 0.05),
             ("spatial_14dof", 30, 1, 0.0), ("spatial_22dof", 600, 400, 0.05), ("xarm6", 150, 0, 0.05),
             ("spatial_18dof", 120, 2500, 0.0)]
    out = []
    for name, n, E, step in specs:
        robot = serve.make_robot(name)
        scene = serve._scene_for(robot, rng, n)
        sid = engine.create_scene(engine.upload_robot(robot), scene)
        D = robot.num_dofs
        q1 = scenes.uniform_configs(rng, E, D)
        u = rng.normal(size=(E, D))
        u /= np.maximum(np.linalg.norm(u, axis=1, keepdims=True), 1e-12)
        q2 = (q1 + u * rng.uniform(0.01, 2.0, (E, 1))).astype(np.float32)
        out.append((robot, scene, sid, q1, q2, step, 10))
    return out


@pytest.mark.parametrize("prec,oracle_prec", [("fp64", "ref64"), ("fp32_ref", "ref32"), ("fp32_recheck", "ref64")])
def test_edges_batch_mixed_robots(engine, prec, oracle_prec):
    """rpm_check_edges_batch: robots of 2-22 DOF, scenes of 8-600 boxes (lane and
    warp layouts in one pipeline), uneven and fixed discretisations and an empty
    item; each item equals the oracle and rpm_check_edges alone."""
    rng = np.random.default_rng(35)
    sets = _edge_items(engine, rng)
    items, outs = [], []
    for robot, scene, sid, q1, q2, step, nc in sets:
        E = q1.shape[0]
        v, k = _t(max(E, 1), torch.uint8), _t(max(E, 1), torch.int32)
        items.append((sid, _t(q1), _t(q2), v, k, step, nc))
        outs.append((v, k))
    engine.check_edges_batch(items, prec)
    engine.sync()
    for (robot, scene, sid, q1, q2, step, nc), (v, k), it in zip(sets, outs, items):
        E = q1.shape[0]
        if E == 0:
            continue
        rv, rk = O.check_edges(robot, scene, q1, q2, step=step, num_checks=nc, prec=oracle_prec)
        assert np.array_equal(v.cpu().numpy()[:E], rv)
        assert np.array_equal(k.cpu().numpy()[:E], rk)
        v1, k1 = _t(E, torch.uint8), _t(E, torch.int32)
        engine.check_edges(sid, it[1], it[2], v1, k1, step=step, num_checks=nc, precision=prec)
        engine.sync()
        assert np.array_equal(v1.cpu().numpy(), rv) and np.array_equal(k1.cpu().numpy(), rk)
    for s in sets:
        engine.destroy_scene(s[2])
