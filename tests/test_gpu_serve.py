"""The serving loop on the GPU: each request's result is the same alone and in
the mix (continuous batching changes scheduling, never results); admission by
memory budget; moving obstacles during a replay."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fresh_outputs(meta):
    return [tuple(None if a is None else a.copy() for a in m[6:]) for m in meta]


def test_alone_equals_mixed(engine):
    """Every kind, DRGBT horizons and motion checks included, gives the same
    bits alone and batched with the others; the DRGBT kinds also equal the
    oracle (spines and motions in the reference's numerics)."""
    from oracle import oracle as O
    from rpmplv2_gb300 import scenes, serve
    wl = serve.serving_workload(engine, seed=41, n_scenes=8, rate=2000.0, duration=0.15, max_size=4096,
                                dynamic_frac=0.5, distinct_outputs=True, drgbt_frac=0.3)
    srv = serve.Server(engine, num_slots=4)
    reqs, meta = wl["requests"], wl["meta"]
    assert len(reqs) > 100
    # alone: one request at a time
    for r in reqs:
        t = srv.wait(srv.submit(r))
        assert t.status == 0 and t.batch_size == 1
    alone = _fresh_outputs(meta)
    kinds = {m[0] for m in meta}
    assert {"valid", "distance", "edges", "reached", "motion"} <= kinds
    # the DRGBT kinds against the oracle (the reference's numerics)
    checked = 0
    for r, m in zip(reqs, meta):
        if m[0] not in ("reached", "motion") or checked >= 12:
            continue
        robot = wl["robots"][wl["scene_robot"][m[3]]]
        sc = wl["scenes"][m[3]]
        if m[0] == "reached":
            qo, st = O.reached_states(robot, sc, m[4], m[5])
            assert np.array_equal(qo.view(np.uint32), m[8].view(np.uint32)) and np.array_equal(st, m[6])
        else:
            box = (serve._abi.MovingBox * max(1, r.num_boxes)).from_address(r.boxes) if r.num_boxes else []
            rv, rk = O.motion_validity(robot, sc, m[4], m[5], box, 0.05, 8, prec="ref32")
            assert np.array_equal(rv, m[6]) and np.array_equal(rk, m[7])
        checked += 1
    assert checked >= 4
    for m in meta:
        for a in m[6:]:
            if a is not None:
                a[:] = 7
    # mixed: all submitted at once, batched and overlapped
    timings = srv.replay(reqs, np.zeros(len(reqs)))
    assert all(t.status == 0 for t in timings)
    assert max(t.batch_size for t in timings) > 1
    for outs, m in zip(alone, meta):
        for a0, a in zip(outs, m[6:]):
            if a0 is not None:
                assert np.array_equal(a0.view(np.uint8), a.view(np.uint8)), m[0]
    srv.close()


def test_admission_by_memory(engine):
    from rpmplv2_gb300 import robots, scenes, serve
    rb = robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    _, sc, q = scenes.xarm6_workload(20000, seed=42)
    sid = engine.create_scene(engine.upload_robot(rb), sc)
    srv = serve.Server(engine, num_slots=2, memory_budget=1 << 20)   # 1 MiB of request buffers
    big = serve.pinned((60000, 6), np.float32)
    vb = serve.pinned(60000, np.uint8)
    t = srv.wait(srv.submit(serve.configs_request(sid, big, vb)))
    assert t.status == -5   # larger than the whole budget: RPM_ERR_ADMISSION
    qs = serve.pinned(q.shape, np.float32)
    qs[:] = q
    reqs, outs = [], []
    for k in range(40):   # 40 x 500 configs = 20,000: more than fits at once
        v = serve.pinned(500, np.uint8)
        outs.append(v)
        reqs.append(serve.configs_request(sid, qs[500 * k:500 * (k + 1)], v))
    timings = srv.replay(reqs, np.zeros(len(reqs)))
    assert all(tm.status == 0 for tm in timings)
    vv, _, _ = engine.check_configs_host(sid, q, "fp32_recheck", want=("valid",))
    assert np.array_equal(np.concatenate(outs), vv)
    srv.close()


def test_moving_obstacles_replay(engine):
    from rpmplv2_gb300 import serve
    wl = serve.serving_workload(engine, seed=43, n_scenes=6, rate=4000.0, duration=0.1, max_size=2048,
                                dynamic_frac=1.0)
    srv = serve.Server(engine, num_slots=4)
    lib = engine.lib
    lib.rpm_scene_info.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.POINTER(ctypes.c_uint64)]
    sid = wl["motions"][0].scene_id
    v0 = ctypes.c_uint64()
    lib.rpm_scene_info(engine.ctx, sid, None, None, ctypes.byref(v0))
    timings = srv.replay(wl["requests"], wl["arrivals"], wl["motions"], period=0.001)
    assert all(t.status == 0 for t in timings)
    v1 = ctypes.c_uint64()
    lib.rpm_scene_info(engine.ctx, sid, None, None, ctypes.byref(v1))
    assert v1.value - v0.value >= 20   # ~1 ms updates during a >= 100 ms replay
    assert all(v0.value <= t.scene_version <= v1.value for t, m in zip(timings, wl["meta"])
               if wl["scene_ids"][m[3]] == sid)
    srv.close()


def test_results_under_moving_obstacles_match_the_oracle(engine):
    """Requests submitted while their scenes' boxes move (DRGBT replanning with
    dynamic obstacles): every result equals the oracle on the scene version the
    request read (rpm_request_timing.scene_version), with versions changing
    between and during the requests' batches."""
    import time
    import torch  # noqa: F401  (pinned buffers)
    from oracle import oracle as O
    from rpmplv2_gb300 import scenes, serve
    rng = np.random.default_rng(44)
    srv = serve.Server(engine, num_slots=4)
    setups = []
    for name, n in (("xarm6", 50), ("spatial_10dof", 120), ("planar_2dof", 12)):
        robot = serve.make_robot(name)
        sc = serve._scene_for(robot, rng, n)
        first = 1 if name == "xarm6" else 0
        mov = rng.choice(np.arange(first, sc.n), size=5, replace=False)
        sc.flags[mov] |= scenes.RPM_OBS_DYNAMIC
        sid = engine.create_scene(engine.upload_robot(robot), sc)
        vel = rng.normal(size=(5, 3)).astype(np.float32)
        vel *= (rng.uniform(0.2, 1.6, (5, 1)) / np.linalg.norm(vel, axis=1, keepdims=True)).astype(np.float32)
        ver = ctypes.c_uint64()
        engine.lib.rpm_scene_info(engine.ctx, sid, None, None, ctypes.byref(ver))
        setups.append({"robot": robot, "scene": sc, "sid": sid, "mov": mov, "vel": vel,
                       "versions": {ver.value: sc.aabb.copy()}})
    pending = []
    for rnd in range(40):
        for st in setups:   # every 1 ms of planner time the dynamic boxes move
            moved = st["scene"].aabb[st["mov"]] + np.tile(st["vel"] * 0.001, 2)
            st["scene"].aabb[st["mov"]] = moved
            ver = engine.update_scene(st["sid"], st["mov"], moved)
            st["versions"][ver] = st["scene"].aabb.copy()
        for _ in range(3):
            st = setups[int(rng.integers(len(setups)))]
            D = st["robot"].num_dofs
            kind = int(rng.integers(3))
            cnt = int(rng.integers(1, 512))
            q = serve.pinned((cnt, D), np.float32)
            q[:] = rng.uniform(-np.pi, np.pi, (cnt, D))
            v = serve.pinned(cnt, np.uint8)
            if kind == 2:
                q2 = serve.pinned((cnt, D), np.float32)
                q2[:] = q + rng.uniform(-0.5, 0.5, (cnt, D))
                k = serve.pinned(cnt, np.int32)
                req = serve.edges_request(st["sid"], q, q2, v, k, step=0.05)
                pending.append((srv.submit(req), st, kind, (q, q2, v, k)))
            else:
                d = serve.pinned(cnt, np.float64) if kind == 1 else None
                req = serve.configs_request(st["sid"], q, v, d)
                pending.append((srv.submit(req), st, kind, (q, v, d)))
        time.sleep(0.0005)
    seen = set()
    for ticket, st, kind, bufs in pending:
        t = srv.wait(ticket)
        assert t.status == 0
        assert t.scene_version in st["versions"], "request read an unknown version"
        seen.add((st["sid"], t.scene_version))
        scene = scenes.Scene(st["versions"][t.scene_version], st["scene"].tol, st["scene"].flags)
        if kind == 2:
            q, q2, v, k = bufs
            rv, rk = O.check_edges(st["robot"], scene, q, q2, step=np.float32(0.05), prec="ref64")
            assert np.array_equal(v, rv) and np.array_equal(k, rk)
        else:
            q, v, d = bufs
            rv, rd, _ = O.check_configs(st["robot"], scene, q, prec="ref64", want=("valid", "dist"))
            assert np.array_equal(v, rv)
            if d is not None:
                assert np.abs(d - rd).max() <= 1e-5
    assert len(seen) >= 10   # requests read many different versions
    srv.close()
    for st in setups:
        engine.destroy_scene(st["sid"])


def test_update_many_scenes_in_one_launch(engine):
    """rpm_scene_update_many writes the next version of several scenes with one
    launch: each scene's checks then equal the oracle on its moved AABBs, and
    a scene listed twice is refused."""
    import torch
    from oracle import oracle as O
    from rpmplv2_gb300 import scenes, serve
    from rpmplv2_gb300.engine import RpmError
    rng = np.random.default_rng(45)
    setups = []
    for name, n in (("xarm6", 40), ("spatial_14dof", 300), ("planar_2dof", 9)):
        robot = serve.make_robot(name)
        sc = serve._scene_for(robot, rng, n)
        sid = engine.create_scene(engine.upload_robot(robot), sc)
        setups.append((robot, sc, sid))
    v0 = [engine.update_scenes([(sid, [], np.zeros((0, 6)))])[0] for _, _, sid in setups]
    ups = []
    for robot, sc, sid in setups:
        first = 1 if robot.name == "xarm6" else 0
        idx = rng.choice(np.arange(first, sc.n), size=min(7, sc.n - first), replace=False).astype(np.int32)
        sc.aabb[idx] += rng.uniform(-0.1, 0.1, (len(idx), 1)).astype(np.float32)
        ups.append((sid, idx, sc.aabb[idx]))
    vers = engine.update_scenes(ups)
    assert vers == [v + 1 for v in v0]
    for robot, sc, sid in setups:
        q = scenes.uniform_configs(rng, 2048, robot.num_dofs)
        v = torch.zeros(2048, dtype=torch.uint8, device="cuda")
        d = torch.zeros(2048, dtype=torch.float64, device="cuda")
        engine.check_configs(sid, torch.from_numpy(q).cuda(), "fp32_recheck", v, d)
        engine.sync()
        rv, rd, _ = O.check_configs(robot, sc, q, prec="ref64", want=("valid", "dist"))
        assert np.array_equal(v.cpu().numpy(), rv) and np.abs(d.cpu().numpy() - rd).max() <= 1e-5
    with pytest.raises(RpmError):
        engine.update_scenes([ups[0], ups[0]])
    for _, _, sid in setups:
        engine.destroy_scene(sid)
