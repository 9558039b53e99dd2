"""GPU parity of the warp-per-configuration layout (obstacles in spatially
sorted leaves, leaf culling, nearest-first distance bands, pair-level FP64
recheck) against the oracle, and its equality with the lane-per-configuration
layout.

Bars as in test_gpu_parity: fp64 and fp32_ref bit-equal to ref64 / ref32,
fp32_recheck with 0 isValid flips and distances within 1e-5 m of ref64.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

pytestmark = pytest.mark.gpu

FORMS = [("fp64", "ref64"), ("fp32_ref", "ref32"), ("fp32_recheck", "ref64")]


@pytest.fixture
def layout(engine):
    yield engine.set_layout
    engine.set_layout("auto")


def _run(engine, sid, q, L, prec, want=("valid", "dist", "profile")):
    C = q.shape[0]
    v = torch.zeros(C, dtype=torch.uint8, device="cuda") if "valid" in want else None
    d = torch.zeros(C, dtype=torch.float64, device="cuda") if "dist" in want else None
    p = torch.zeros((C, L), dtype=torch.float32, device="cuda") if "profile" in want else None
    engine.check_configs(sid, torch.from_numpy(q).cuda(), prec, v, d, p)
    engine.sync()
    return tuple(x.cpu().numpy() if x is not None else None for x in (v, d, p))


def _assert_oracle(robot, scene, q, out, prec, oprec, want=("valid", "dist", "profile")):
    rv, rd, rp = O.check_configs(robot, scene, q, prec=oprec, want=want)
    v, d, p = out
    if v is not None:
        assert np.array_equal(v, rv), "%s: %d isValid flips" % (prec, int((v != rv).sum()))
    if prec == "fp32_recheck":
        if d is not None:
            assert np.abs(d - rd).max() <= 1e-5
        if p is not None:
            assert np.abs(p.astype(np.float64) - rp).max() <= 2e-5
    else:
        if d is not None:
            assert np.array_equal(d.view(np.uint64), rd.view(np.uint64))
        if p is not None:
            assert np.array_equal(p.view(np.uint32), rp.view(np.uint32))


def _big_scene(seed, n, dim_lo, dim_hi, radius, tol=None):
    rng = np.random.default_rng(seed)
    boxes = [scenes.box_aabb(rng.uniform(dim_lo, dim_hi, 3), c) for c in
             scenes._ball(rng, n, scenes.SPATIAL_WS_CENTER, radius)]
    t = None if tol is None else rng.uniform(tol[0], tol[1], n).astype(np.float32)
    return scenes.Scene(np.array(boxes), tol=t)


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_warp_xarm6(engine, layout, prec, oprec):
    robot, scene, q = scenes.xarm6_workload(8192, seed=41)
    layout("warp")
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    out = _run(engine, sid, q, robot.num_links, prec)
    engine.destroy_scene(sid)
    _assert_oracle(robot, scene, q, out, prec, oprec)


@pytest.mark.parametrize("prec,oprec", FORMS)
@pytest.mark.parametrize("dense", [True, False])
def test_warp_big_scene_matches_lane(engine, layout, prec, oprec, dense):
    """1000 boxes, 18 links: dense (most configurations collide) and sparse
    (distances found by the nearest-first search)."""
    robot = robots.spatial(18, radius=0.03)
    scene = _big_scene(42, 1000, 0.02, 0.15, 1.5) if dense else _big_scene(43, 1000, 0.005, 0.02, 2.5)
    q = scenes.uniform_configs(np.random.default_rng(44), 1536, 18)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    layout("warp")
    wide = _run(engine, sid, q, robot.num_links, prec)
    layout("lane")
    lane = _run(engine, sid, q, robot.num_links, prec)
    engine.destroy_scene(sid)
    _assert_oracle(robot, scene, q, wide, prec, oprec)
    if prec != "fp32_recheck":
        for a, b in zip(wide, lane):
            assert np.array_equal(a, b)
    else:
        assert np.array_equal(wide[0], lane[0])


@pytest.mark.parametrize("want", [("valid",), ("dist",), ("profile",), ("valid", "dist")])
def test_warp_partial_outputs(engine, layout, want):
    robot = robots.spatial(14, radius=0.03)
    scene = _big_scene(45, 600, 0.01, 0.06, 2.0)
    q = scenes.uniform_configs(np.random.default_rng(46), 1024, 14)
    layout("warp")
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    for prec, oprec in (("fp64", "ref64"), ("fp32_recheck", "ref64")):
        out = _run(engine, sid, q, robot.num_links, prec, want)
        _assert_oracle(robot, scene, q, out, prec, oprec, want)
    engine.destroy_scene(sid)


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_warp_ground_and_tolerances(engine, layout, prec, oprec):
    """xArm6 with the ground skipped for its first links, 300 boxes whose
    min_dist_tol varies (the clamp of computeDistance, :367-368)."""
    robot = robots.xarm6(radius=0.05, gripper_length=0.1)
    big = _big_scene(47, 300, 0.02, 0.08, 1.0, tol=(0.005, 0.3))
    g, gt = scenes.ground_box()
    aabb = np.vstack([big.aabb[:120], g[None, :], big.aabb[120:]])
    tol = np.concatenate([big.tol[:120], [gt], big.tol[120:]]).astype(np.float32)
    flags = np.zeros(aabb.shape[0], np.uint8)
    flags[120] = 1
    scene = scenes.Scene(aabb, tol=tol, flags=flags)
    q = scenes.uniform_configs(np.random.default_rng(48), 4096, 6)
    layout("warp")
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    out = _run(engine, sid, q, robot.num_links, prec)
    engine.destroy_scene(sid)
    _assert_oracle(robot, scene, q, out, prec, oprec)


def test_warp_empty_scene(engine, layout):
    robot = robots.spatial(10, radius=0.03)
    scene = scenes.Scene(np.zeros((0, 6), np.float32))
    q = scenes.uniform_configs(np.random.default_rng(49), 100, 10)
    layout("warp")
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    for prec, oprec in FORMS:
        out = _run(engine, sid, q, robot.num_links, prec)
        assert out[0].min() == 1 and np.all(out[1] == 1000.0) and np.all(out[2] == 1000.0)
        _assert_oracle(robot, scene, q, out, prec, oprec)
    engine.destroy_scene(sid)


@pytest.mark.parametrize("count", [1, 7, 33, 257, 3001])
def test_warp_ragged_counts(engine, layout, count):
    robot = robots.spatial(22, radius=0.03)
    scene = _big_scene(50, 500, 0.02, 0.15, 1.5)
    q = scenes.uniform_configs(np.random.default_rng(51 + count), count, 22)
    layout("warp")
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    out = _run(engine, sid, q, robot.num_links, "fp64")
    engine.destroy_scene(sid)
    _assert_oracle(robot, scene, q, out, "fp64", "ref64")


def test_warp_after_incremental_update(engine, layout):
    """Moved obstacles reach the sorted copy: the next version is checked
    against the oracle on the moved scene, in both layouts."""
    robot = robots.spatial(14, radius=0.03)
    scene = _big_scene(52, 800, 0.02, 0.1, 1.5)
    rng = np.random.default_rng(53)
    q = scenes.uniform_configs(rng, 2048, 14)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    idx = rng.choice(scene.n, 64, replace=False).astype(np.int32)
    moved = scene.aabb[idx] + rng.uniform(-0.3, 0.3, (64, 1)).astype(np.float32)
    engine.update_scene(sid, idx, moved)
    aabb = scene.aabb.copy()
    aabb[idx] = moved
    new_scene = scenes.Scene(aabb, tol=scene.tol, flags=scene.flags)
    for lay in ("warp", "lane"):
        layout(lay)
        out = _run(engine, sid, q, robot.num_links, "fp64")
        _assert_oracle(robot, new_scene, q, out, "fp64", "ref64")
    engine.destroy_scene(sid)


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_auto_batch_mixes_layouts(engine, layout, prec, oprec):
    """One batch holding a small scene (lane layout) and a large one (warp
    layout): both segments match the oracle."""
    layout("auto")
    r_small, s_small, q_small = scenes.xarm6_workload(4096, seed=54)
    r_big = robots.spatial(18, radius=0.03)
    s_big = _big_scene(55, 700, 0.02, 0.12, 1.5)
    q_big = scenes.uniform_configs(np.random.default_rng(56), 2048, 18)
    parts, items = [], []
    for robot, scene, q in ((r_small, s_small, q_small), (r_big, s_big, q_big)):
        sid = engine.create_scene(engine.upload_robot(robot), scene)
        C, L = q.shape[0], robot.num_links
        v = torch.zeros(C, dtype=torch.uint8, device="cuda")
        d = torch.zeros(C, dtype=torch.float64, device="cuda")
        p = torch.zeros((C, L), dtype=torch.float32, device="cuda")
        items.append((sid, torch.from_numpy(q).cuda(), v, d, p))
        parts.append((robot, scene, q, v, d, p))
    engine.check_batch(items, prec)
    engine.sync()
    for robot, scene, q, v, d, p in parts:
        _assert_oracle(robot, scene, q, (v.cpu().numpy(), d.cpu().numpy(), p.cpu().numpy()), prec, oprec)
    for it in items:
        engine.destroy_scene(it[0])


@pytest.mark.parametrize("prec,oprec", FORMS)
def test_warp_edges_match_oracle_and_lane(engine, layout, prec, oprec):
    """isValid(q1, q2) batches with uneven discretisation: the warp-per-check
    pass gives the reference's validity and check counts, as the lane pass does."""
    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(4000, seed=57)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    outs = {}
    for lay in ("warp", "lane"):
        layout(lay)
        v = torch.zeros(q1.shape[0], dtype=torch.uint8, device="cuda")
        k = torch.zeros(q1.shape[0], dtype=torch.int32, device="cuda")
        engine.check_edges(sid, torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda(), v, k, step=float(step),
                           precision=prec)
        engine.sync()
        outs[lay] = (v.cpu().numpy(), k.cpu().numpy())
    engine.destroy_scene(sid)
    rv, rk = O.check_edges(robot, scene, q1, q2, step=step, prec=oprec)
    assert np.array_equal(outs["warp"][0], rv) and np.array_equal(outs["warp"][1], rk)
    assert np.array_equal(outs["lane"][0], rv) and np.array_equal(outs["lane"][1], rk)


@pytest.mark.parametrize("prec,oprec", FORMS)
@pytest.mark.parametrize("n", [100, 700])
def test_lane_edges_staged_rows(engine, layout, prec, oprec, n):
    """The lane edge pass with one scene staged in shared memory: read through
    the per-obstacle copy of the rows (100 boxes) and through the plain rows
    (700 boxes, beyond the copy's size limit)."""
    robot = robots.spatial(10, radius=0.03)
    scene = _big_scene(61 + n, n, 0.02, 0.08, 1.4)
    rng = np.random.default_rng(62)
    q1 = scenes.uniform_configs(rng, 400, 10)
    q2 = (q1 + rng.uniform(-0.6, 0.6, q1.shape)).astype(np.float32)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    layout("lane")
    v = torch.zeros(400, dtype=torch.uint8, device="cuda")
    k = torch.zeros(400, dtype=torch.int32, device="cuda")
    engine.check_edges(sid, torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda(), v, k, step=0.05,
                       precision=prec)
    engine.sync()
    engine.destroy_scene(sid)
    rv, rk = O.check_edges(robot, scene, q1, q2, step=0.05, prec=oprec)
    assert np.array_equal(v.cpu().numpy(), rv) and np.array_equal(k.cpu().numpy(), rk)
    assert 0 < int(rv.sum()) < 400


def test_warp_edges_big_scene_fixed_count(engine, layout):
    """22 links against 1000 boxes with the fixed NUM_INTERPOLATION_VALIDITY_CHECKS
    discretisation (step <= 0), FP32 + FP64 recheck, with CUDA-graph replay."""
    robot = robots.spatial(22, radius=0.03)
    scene = _big_scene(58, 1000, 0.01, 0.06, 2.0)
    rng = np.random.default_rng(59)
    q1 = scenes.uniform_configs(rng, 600, 22)
    q2 = (q1 + rng.uniform(-0.3, 0.3, q1.shape)).astype(np.float32)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    layout("warp")
    engine.set_graphs(True)
    try:
        for _ in range(2):   # capture, then replay
            v = torch.zeros(600, dtype=torch.uint8, device="cuda")
            k = torch.zeros(600, dtype=torch.int32, device="cuda")
            engine.check_edges(sid, torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda(), v, k, step=0.0,
                               num_checks=10, precision="fp32_recheck")
            engine.sync()
            rv, rk = O.check_edges(robot, scene, q1, q2, step=0.0, num_checks=10, prec="ref64")
            assert np.array_equal(v.cpu().numpy(), rv) and np.array_equal(k.cpu().numpy(), rk)
    finally:
        engine.set_graphs(False)
        engine.destroy_scene(sid)


def test_maximum_scene_size(engine):
    """RPM_MAX_OBSTACLES boxes: every layout and form against the oracle (the
    pair-recheck entries index obstacles up to 2047); one more is refused."""
    from rpmplv2_gb300 import robots
    from rpmplv2_gb300.engine import RpmError
    rng = np.random.default_rng(97)
    rb = robots.spatial(14, radius=0.03)
    n = 2048
    boxes = [scenes.box_aabb(rng.uniform(0.01, 0.04, 3), c) for c in scenes._ball(rng, n, scenes.SPATIAL_WS_CENTER, 1.5)]
    sc = scenes.Scene(np.array(boxes), tol=rng.uniform(0.2, 2.0, n).astype(np.float32))
    q = scenes.uniform_configs(rng, 3000, 14)
    sid = engine.create_scene(engine.upload_robot(rb), sc)
    rv64, rd64, _ = O.check_configs(rb, sc, q, prec="ref64")
    for layout in ("lane", "warp"):
        engine.set_layout(layout)
        for prec in ("fp64", "fp32_recheck"):
            v = torch.zeros(q.shape[0], dtype=torch.uint8, device="cuda")
            d = torch.zeros(q.shape[0], dtype=torch.float64, device="cuda")
            engine.check_configs(sid, torch.from_numpy(q).cuda(), prec, v, d, None)
            engine.sync()
            assert np.array_equal(v.cpu().numpy(), rv64), (layout, prec)
            err = np.abs(d.cpu().numpy() - rd64).max()
            assert err <= (1e-9 if prec == "fp64" else 1e-5), (layout, prec, err)
    engine.set_layout("auto")
    engine.destroy_scene(sid)
    big = scenes.Scene(np.concatenate([sc.aabb, sc.aabb[:1]]))
    with pytest.raises(RpmError):
        engine.create_scene(engine.upload_robot(rb), big)
