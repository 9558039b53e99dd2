"""The serving loop on the GPU: each request's result is the same alone and in
the mix (continuous batching changes scheduling, never results); admission by
memory budget; moving obstacles during a replay."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fresh_outputs(meta):
    return [(m[6].copy(), None if m[7] is None else m[7].copy()) for m in meta]


def test_alone_equals_mixed(engine):
    from rpmplv2_gb300 import serve
    wl = serve.serving_workload(engine, seed=41, n_scenes=8, rate=2000.0, duration=0.15, max_size=4096,
                                dynamic_frac=0.0, distinct_outputs=True)
    srv = serve.Server(engine, num_slots=4)
    reqs, meta = wl["requests"], wl["meta"]
    assert len(reqs) > 100
    # alone: one request at a time
    for r in reqs:
        t = srv.wait(srv.submit(r))
        assert t.status == 0 and t.batch_size == 1
    alone = _fresh_outputs(meta)
    for m in meta:
        m[6][:] = 9
        if m[7] is not None:
            m[7][:] = -1
    # mixed: all submitted at once, batched and overlapped
    timings = srv.replay(reqs, np.zeros(len(reqs)))
    assert all(t.status == 0 for t in timings)
    assert max(t.batch_size for t in timings) > 1
    for (v0, d0), m in zip(alone, meta):
        assert np.array_equal(v0, m[6])
        if d0 is not None:
            assert np.array_equal(d0.view(np.uint8), m[7].view(np.uint8))
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
    srv.close()
