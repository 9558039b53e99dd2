"""rpm_check_configs_noalloc against rpm_check_configs.

The no-allocation entry point serves callers that cannot call cudaMalloc (a
real-time loop that forbids allocator calls after start-up, or a framework
that owns all device memory).  It keeps its recheck list
in a static device array shared by every call, so this test makes two calls in
a row on different inputs and checks each against the allocating entry point
with the FP32 + FP64-recheck tolerance of the parity tests: isValid identical,
distances within 1e-5 m.  The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, robot, scene_dev, q, valid, dist, prof):
    import torch
    from rpmplv2_gb300._abi import Params
    aabb, tol, flags, n = scene_dev
    params = Params(1e-4, 1000.0)
    rc = lib.rpm_check_configs_noalloc(ctypes.addressof(robot.desc), aabb.data_ptr(), tol.data_ptr(), flags.data_ptr(),
                                       n, ctypes.byref(params), q.data_ptr(), q.shape[0], valid.data_ptr(),
                                       dist.data_ptr(), prof.data_ptr(), None)
    assert rc == 0, lib.rpm_last_error_string().decode()
    torch.cuda.synchronize()


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rpmplv2_gb300 import scenes
    from rpmplv2_gb300.engine import Engine

    eng = Engine(0)
    lib = eng.lib
    for seed in (21, 22):   # two calls in a row share the static scratch array
        robot, scene, q = scenes.xarm6_workload(40000, seed=seed)
        C, L = q.shape[0], robot.num_links
        rid = eng.upload_robot(robot)
        sid = eng.create_scene(rid, scene)
        qd = torch.from_numpy(q).cuda()
        v_ref = torch.zeros(C, dtype=torch.uint8, device="cuda")
        d_ref = torch.zeros(C, dtype=torch.float64, device="cuda")
        p_ref = torch.zeros((C, L), dtype=torch.float32, device="cuda")
        eng.check_configs(sid, qd, "fp32_recheck", v_ref, d_ref, p_ref)
        eng.sync()
        scene_dev = (torch.from_numpy(scene.aabb).cuda(), torch.from_numpy(scene.tol).cuda(),
                     torch.from_numpy(scene.flags).cuda(), scene.n)
        v = torch.full((C,), 7, dtype=torch.uint8, device="cuda")
        d = torch.full((C,), -1.0, dtype=torch.float64, device="cuda")
        p = torch.full((C, L), -1.0, dtype=torch.float32, device="cuda")
        _noalloc(lib, robot, scene_dev, qd, v, d, p)
        assert torch.equal(v, v_ref), "isValid differs in %d configurations" % int((v != v_ref).sum())
        assert float((d - d_ref).abs().max()) <= 1e-5
        assert float((p - p_ref).abs().max()) <= 1e-5
        eng.destroy_scene(sid)
    # sizes beyond the static array's capacity are rejected, not truncated
    big = torch.zeros((65537, 6), dtype=torch.float32, device="cuda")
    out_v = torch.zeros(65537, dtype=torch.uint8, device="cuda")
    from rpmplv2_gb300._abi import Params, RPM_ERR_RANGE
    rc = lib.rpm_check_configs_noalloc(ctypes.addressof(robot.desc), scene_dev[0].data_ptr(), None, None, scene.n,
                                       ctypes.byref(Params(1e-4, 1000.0)), big.data_ptr(), 65537, out_v.data_ptr(),
                                       None, None, None)
    assert rc == RPM_ERR_RANGE
    assert b"65536" in lib.rpm_last_error_string()
    eng.close()


def test_noalloc_defaults_and_empty_inputs():
    """min_dist_tol and flags may be NULL (MAX_DISTANCE and no ground, as
    rpm_scene_create takes them); an empty obstacle set needs no array; an
    empty batch is a no-op."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rpmplv2_gb300 import robots, scenes
    from rpmplv2_gb300._abi import Params
    from rpmplv2_gb300.engine import Engine

    eng = Engine(0)
    lib = eng.lib
    robot = robots.spatial(10, radius=0.03)
    _, sc, q = scenes.spatial10_edge_workload(2048, seed=23)[:3]
    q = np.ascontiguousarray(q)
    plain = scenes.Scene(sc.aabb)   # no tolerances, no flags
    C = q.shape[0]
    qd = torch.from_numpy(q).cuda()
    for scene, n in ((plain, plain.n), (scenes.Scene(np.zeros((0, 6), np.float32)), 0)):
        sid = eng.create_scene(eng.upload_robot(robot), scene)
        v_ref = torch.zeros(C, dtype=torch.uint8, device="cuda")
        d_ref = torch.zeros(C, dtype=torch.float64, device="cuda")
        eng.check_configs(sid, qd, "fp32_recheck", v_ref, d_ref, None)
        eng.sync()
        aabb = torch.from_numpy(scene.aabb).cuda() if n else None
        v = torch.full((C,), 7, dtype=torch.uint8, device="cuda")
        d = torch.full((C,), -1.0, dtype=torch.float64, device="cuda")
        rc = lib.rpm_check_configs_noalloc(ctypes.addressof(robot.desc), aabb.data_ptr() if n else None, None, None,
                                           n, ctypes.byref(Params(1e-4, 1000.0)), qd.data_ptr(), C, v.data_ptr(),
                                           d.data_ptr(), None, None)
        assert rc == 0, lib.rpm_last_error_string().decode()
        torch.cuda.synchronize()
        assert torch.equal(v, v_ref)
        assert float((d - d_ref).abs().max()) <= 1e-5
        eng.destroy_scene(sid)
    rc = lib.rpm_check_configs_noalloc(ctypes.addressof(robot.desc), None, None, None, 0,
                                       ctypes.byref(Params(1e-4, 1000.0)), None, 0, None, None, None, None)
    assert rc == 0
    eng.close()
