"""Python front end of the serving loop (rpm_server_* in include/rpm_gpu.h) and
the serving workload: resident scenes from the reference's robots, moving
obstacles, and a Poisson trace of mixed-size isValid / distance / edge
requests (DRGBT-style replanning traffic from many planners)."""
import ctypes
import math

import numpy as np

from . import _abi  # noqa: F401
from . import robots as _robots
from . import scenes as _scenes
from .engine import _check, _i32, _i64, _vp, load

RPM_REQ_CONFIGS = 0
RPM_REQ_EDGES = 1
RPM_REQ_REACHED = 2
RPM_REQ_MOTION = 3


class ServerConfig(ctypes.Structure):
    _fields_ = [("num_slots", ctypes.c_int32), ("precision", ctypes.c_int32), ("memory_budget", ctypes.c_int64),
                ("max_batch_segments", ctypes.c_int32), ("max_batch_configs", ctypes.c_int32),
                ("express_slots", ctypes.c_int32), ("express_work", ctypes.c_int32), ("chunk_work", ctypes.c_int32),
                ("bulk_sms", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("scene_id", ctypes.c_int32), ("count", ctypes.c_int64),
                ("q_host", ctypes.c_void_p), ("q1_host", ctypes.c_void_p), ("q2_host", ctypes.c_void_p),
                ("step", ctypes.c_float), ("num_checks", ctypes.c_int32), ("valid_host", ctypes.c_void_p),
                ("dist_host", ctypes.c_void_p), ("profile_host", ctypes.c_void_p), ("checks_host", ctypes.c_void_p),
                ("spine", ctypes.c_void_p), ("q_out_host", ctypes.c_void_p), ("status_host", ctypes.c_void_p),
                ("boxes", ctypes.c_void_p), ("num_boxes", ctypes.c_int32), ("num_points", ctypes.c_int32),
                ("max_iter_time", ctypes.c_float), ("reserved", ctypes.c_int32)]


class Timing(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("batch_size", ctypes.c_int32), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_launch", ctypes.c_double), ("t_done", ctypes.c_double),
                ("scene_version", ctypes.c_uint64), ("h2d_ms", ctypes.c_float), ("kernel_ms", ctypes.c_float),
                ("d2h_ms", ctypes.c_float), ("enqueue_ms", ctypes.c_float)]


class Motion(ctypes.Structure):
    _fields_ = [("scene_id", ctypes.c_int32), ("index", ctypes.c_int32), ("velocity", ctypes.c_float * 3)]


def _bind(L):
    if getattr(L, "_rpm_server_bound", False):
        return
    L.rpm_server_create.argtypes = [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]
    L.rpm_server_submit.argtypes = [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]
    L.rpm_server_poll.argtypes = [_vp, ctypes.c_uint64, ctypes.POINTER(Timing)]
    L.rpm_server_wait.argtypes = [_vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(Timing)]
    L.rpm_server_release.argtypes = [_vp, ctypes.c_uint64]
    L.rpm_server_replay.argtypes = [_vp, _vp, _vp, _i64, _vp, _i32, ctypes.c_double, _vp]
    L.rpm_server_stats.argtypes = [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.rpm_server_destroy.argtypes = [_vp]
    L._rpm_server_bound = True


def _addr(a):
    return None if a is None else a.ctypes.data


def pinned(shape, dtype):
    """A numpy array in page-locked host memory (copies to and from it
    overlap); plain host memory where no CUDA driver is present.  The array's
    base is the pinned torch tensor, which keeps the storage alive."""
    import torch
    dt = {np.float32: torch.float32, np.float64: torch.float64, np.uint8: torch.uint8,
          np.int32: torch.int32}[np.dtype(dtype).type]
    t = torch.empty(shape, dtype=dt)
    if torch.cuda.is_available():
        t = t.pin_memory()
    return t.numpy()


class Server:
    def __init__(self, engine, num_slots=0, precision="fp32_recheck", memory_budget=8 << 30, max_batch_segments=32,
                 max_batch_configs=0, express_slots=0, express_work=0, chunk_work=0, bulk_sms=0):
        """num_slots bulk streams, express_slots high-priority streams, and
        optionally an SM partition of bulk_sms SMs for the bulk streams; 0
        takes the library's defaults (rpm_server_config)."""
        from ._abi import PRECISIONS
        self.engine = engine
        self.lib = load()
        _bind(self.lib)
        cfg = ServerConfig(num_slots, PRECISIONS[precision], memory_budget, max_batch_segments, max_batch_configs,
                           express_slots, express_work, chunk_work, bulk_sms, 0)
        self.srv = _vp()
        _check(self.lib.rpm_server_create(engine.ctx, ctypes.byref(cfg), ctypes.byref(self.srv)))

    def close(self):
        if self.srv:
            self.lib.rpm_server_destroy(self.srv)
            self.srv = _vp()

    def submit(self, req):
        t = ctypes.c_uint64()
        _check(self.lib.rpm_server_submit(self.srv, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def wait(self, ticket, timeout=120.0):
        tm = Timing()
        rc = self.lib.rpm_server_wait(self.srv, ticket, timeout, ctypes.byref(tm))
        self.lib.rpm_server_release(self.srv, ticket)
        _check(rc)
        return tm

    def replay(self, reqs, arrivals, motions=(), period=0.0):
        n = len(reqs)
        arr = (Request * n)(*reqs)
        ts = np.ascontiguousarray(arrivals, np.float64)
        mot = (Motion * max(1, len(motions)))(*motions) if motions else None
        out = (Timing * n)()
        _check(self.lib.rpm_server_replay(self.srv, ctypes.addressof(arr), ts.ctypes.data, n,
                                          ctypes.addressof(mot) if mot is not None else None, len(motions),
                                          float(period), ctypes.addressof(out)))
        return [out[i] for i in range(n)]

    def stats(self):
        b, p = ctypes.c_int64(), ctypes.c_int64()
        _check(self.lib.rpm_server_stats(self.srv, ctypes.byref(b), ctypes.byref(p)))
        return {"batches": b.value, "pending": p.value}


def configs_request(scene_id, q, valid=None, dist=None, profile=None):
    return Request(RPM_REQ_CONFIGS, scene_id, q.shape[0], _addr(q), None, None, 0.0, 0, _addr(valid), _addr(dist),
                   _addr(profile), None)


def edges_request(scene_id, q1, q2, valid, checks=None, step=0.05, num_checks=10):
    return Request(RPM_REQ_EDGES, scene_id, q1.shape[0], None, _addr(q1), _addr(q2), step, num_checks, _addr(valid),
                   None, None, _addr(checks))


def reached_request(scene_id, q_current, horizon, q_out, status, spine, dist=None):
    """DRGBT::computeReachedState over a horizon (rpm_reached_states); spine
    is an rpm_spine_params (kept alive by the caller)."""
    return Request(RPM_REQ_REACHED, scene_id, horizon.shape[0], _addr(q_current), _addr(horizon), None, 0.0, 0,
                   None, _addr(dist), None, None, ctypes.addressof(spine), _addr(q_out), _addr(status))


def motion_request(scene_id, q_prev, q_cur, valid, boxes, max_iter_time, num_points, checks=None):
    """MotionValidity::check with moving boxes (rpm_motion_validity); boxes is
    a ctypes array of rpm_moving_box (kept alive by the caller)."""
    return Request(RPM_REQ_MOTION, scene_id, q_prev.shape[0], None, _addr(q_prev), _addr(q_cur), 0.0, 0,
                   _addr(valid), None, None, _addr(checks), None, None, None,
                   ctypes.addressof(boxes) if len(boxes) else None, len(boxes), int(num_points), float(max_iter_time))


# ----------------------------------------------------------------- workload --
def reject_touching(robot, aabbs, margin=0.01, samples=33):
    """Mask of boxes that stay clear of the capsule skeleton at q = 0 (the
    reference's generator drops obstacles that invalidate the start)."""
    sk = robot.skeleton_np(np.zeros(robot.num_dofs))
    t = np.linspace(0.0, 1.0, samples)
    pts = sk[:-1, None, :] + t[None, :, None] * (sk[1:] - sk[:-1])[:, None, :]        # (L, S, 3)
    seg_len = np.linalg.norm(sk[1:] - sk[:-1], axis=1) / (samples - 1)
    lo, hi = aabbs[:, None, None, :3], aabbs[:, None, None, 3:]
    d = np.maximum(np.maximum(lo - pts[None], pts[None] - hi), 0.0)
    dist = np.sqrt((d * d).sum(-1)).min(-1)                                              # (n, L)
    need = robot.capsule_radius[None, :] + margin + seg_len[None, :]
    return (dist > need).all(1)


def _scene_for(robot, rng, n):
    if robot.name == "planar_2dof":
        dims = rng.uniform(0.1, 0.5, (n, 2))
        rr, th = 2.0 * np.sqrt(rng.uniform(size=n)), rng.uniform(0, 2 * math.pi, n)
        c = np.stack([rr * np.cos(th), rr * np.sin(th), np.zeros(n)], 1)
        h = np.concatenate([dims / 2, np.full((n, 1), 0.05)], 1)
        return _scenes.Scene(np.concatenate([c - h, c + h], 1).astype(np.float32))
    if robot.name == "xarm6":
        boxes, g_aabb, g_tol = [], *_scenes.ground_box()
        center, radius, half = np.array([0.0, 0.0, 0.267]), 1.0, 0.025
    else:
        boxes, center, radius = [], np.array(_scenes.SPATIAL_WS_CENTER), 1.2
    out = np.zeros((0, 6), np.float32)
    while out.shape[0] < n:
        m = 2 * (n - out.shape[0]) + 8
        p = rng.uniform(-1, 1, (m, 3))
        c = center + radius * p[(p * p).sum(1) <= 1.0]
        hh = np.full((c.shape[0], 3), half) if robot.name == "xarm6" else rng.uniform(0.01, 0.05, (c.shape[0], 3))
        cand = np.concatenate([c - hh, c + hh], 1).astype(np.float32)
        out = np.concatenate([out, cand[reject_touching(robot, cand)]])[:n]
    if robot.name == "xarm6":
        aabb = np.concatenate([g_aabb[None, :], out])
        tol = np.full(n + 1, _scenes.MAX_DISTANCE, np.float32)
        tol[0] = g_tol
        flags = np.zeros(n + 1, np.uint8)
        flags[0] = 1
        return _scenes.Scene(aabb, tol, flags)
    return _scenes.Scene(out)


SERVE_ROBOTS = ("planar_2dof", "xarm6", "spatial_10dof", "spatial_14dof", "spatial_18dof", "spatial_22dof")


def make_robot(name):
    if name == "planar_2dof":
        return _robots.planar_2dof(radius=0.0)
    if name == "xarm6":
        return _robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    return _robots.by_name(name, radius=0.03)


def serving_workload(engine, seed=4, n_scenes=64, rate=20000.0, duration=0.5, max_size=65536, dynamic_frac=0.2,
                     n_dynamic=5, max_speed=1.6, edge_divisor=16, pool=65536, distinct_outputs=False, drgbt_frac=0.1):
    """Scenes on the device, a Poisson request trace and the moving obstacles.

    Request sizes are log-uniform in [1, max_size]; kinds are isValid,
    isValid + computeDistance and edge checks in equal shares.  An edge
    request of size s carries max(1, s // edge_divisor) edges at 0.05 rad
    steps (about 12 checks each), so its work is near a configuration
    request of the same size.  A drgbt_frac share of the requests are DRGBT
    replanning steps instead (DRGBT.cpp:79-176): half a horizon of reached
    states (10 + 2D - 2 states, DRGBT.cpp:24-25; 5 layers, NUM_ITER_SPINE 1,
    expanded bubble, D_CRIT 0.05) with the reached states' distances, half a
    MotionValidity::check of 1-16 motions at 8 points while the scene's
    dynamic boxes move straight (MotionValidity.cpp:30-53).  Inputs are
    slices of per-DOF pinned pools; outputs alias shared pinned pools unless
    distinct_outputs is set."""
    rng = np.random.default_rng(seed)
    robots = {name: make_robot(name) for name in SERVE_ROBOTS}
    rids = {name: engine.upload_robot(r) for name, r in robots.items()}
    scene_ids, scene_robot, scene_n, motions, sc_aabb = [], [], [], [], []
    for s in range(n_scenes):
        name = SERVE_ROBOTS[rng.integers(len(SERVE_ROBOTS))]
        n = int(round(math.exp(rng.uniform(math.log(10), math.log(1000)))))
        sc = _scene_for(robots[name], rng, n)
        moving = []
        if rng.uniform() < dynamic_frac:
            first = 1 if name == "xarm6" else 0
            moving = rng.choice(np.arange(first, sc.n), size=min(n_dynamic, sc.n - first), replace=False)
            sc.flags[moving] |= _scenes.RPM_OBS_DYNAMIC   # label "dynamic_obstacle"
        sid = engine.create_scene(rids[name], sc)
        scene_ids.append(sid)
        scene_robot.append(name)
        scene_n.append(sc.n)
        sc_aabb.append(_scenes.Scene(sc.aabb.copy(), sc.tol.copy(), sc.flags.copy()))
        for j in moving:
            u = rng.normal(size=3)
            u = u / np.linalg.norm(u) * rng.uniform(0, max_speed)
            motions.append(Motion(sid, int(j), (ctypes.c_float * 3)(*u)))
    dofs = sorted({robots[n].num_dofs for n in SERVE_ROBOTS})
    qpool = {d: pinned((pool, d), np.float32) for d in dofs}
    q2pool = {}
    for d in dofs:
        qpool[d][:] = rng.uniform(-math.pi, math.pi, (pool, d))
        u = rng.normal(size=(pool, d))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        q2pool[d] = pinned((pool, d), np.float32)
        q2pool[d][:] = qpool[d] + u * rng.uniform(0.01, 2.0, (pool, 1))
    shared = {"valid": pinned(pool, np.uint8), "dist": pinned(pool, np.float64), "checks": pinned(pool, np.int32)}
    n_req = rng.poisson(rate * duration)
    arrivals = np.sort(rng.uniform(0, duration, n_req))
    reqs, meta, keep = [], [], []
    from ._abi import MovingBox, SpineParams
    spine = SpineParams(5, 1, 1, 0.05)
    keep.append(spine)
    movers = {}   # scene index -> rpm_moving_box array of its dynamic boxes (straight motion along -x)
    for s in range(n_scenes):
        sid = scene_ids[s]
        mv = [m for m in motions if m.scene_id == sid]
        arr = (MovingBox * max(1, len(mv)))()
        for k, m in enumerate(mv):
            lo, hi = sc_aabb[s].aabb[m.index, :3], sc_aabb[s].aabb[m.index, 3:]
            arr[k] = MovingBox(m.index, float(np.linalg.norm(np.array(m.velocity[:]))), tuple((hi - lo).tolist()),
                               tuple(((lo + hi) / 2).tolist()), (0.0, 0.0, 0.0, 1.0))
        movers[s] = (arr, len(mv))
        keep.append(arr)
    for i in range(n_req):
        s = int(rng.integers(n_scenes))
        name = scene_robot[s]
        d = robots[name].num_dofs
        size = int(min(max_size, round(math.exp(rng.uniform(0, math.log(max_size))))))
        kind = int(rng.integers(3))
        if rng.uniform() < drgbt_frac:
            kind = 3 + int(rng.integers(2))
        off = int(rng.integers(0, pool - size + 1))
        if kind == 3:   # a DRGBT horizon
            H = 10 + 2 * d - 2
            off = int(rng.integers(0, pool - H - 1))
            qc, hz = qpool[d][off:off + 1], qpool[d][off + 1:off + 1 + H]
            qo = pinned((H, d), np.float32)
            st = pinned(H, np.int32)
            dd = pinned(H, np.float64)
            reqs.append(reached_request(scene_ids[s], qc, hz, qo, st, spine, dd))
            keep += [qo, st, dd]
            meta.append(("reached", 64 * H, 64 * H, s, qc, hz, st, dd, qo))
            continue
        if kind == 4:   # MotionValidity::check while the dynamic boxes move
            M = int(rng.integers(1, 17))
            off = int(rng.integers(0, pool - M + 1))
            arr, nb = movers[s]
            q1 = qpool[d][off:off + M]
            q2 = (q1 + rng.uniform(-0.3, 0.3, q1.shape)).astype(np.float32)
            q2p = pinned((M, d), np.float32)
            q2p[:] = q2
            v = pinned(M, np.uint8)
            k = pinned(M, np.int32)
            reqs.append(motion_request(scene_ids[s], q1, q2p, v, arr if nb else (MovingBox * 0)(), 0.05, 8, k))
            keep += [q2p, v, k]
            meta.append(("motion", 8 * M, 8 * M, s, q1, q2p, v, k))
            continue
        if kind == 2:
            ne = max(1, size // edge_divisor)
            off = int(rng.integers(0, pool - ne + 1))
            v = pinned(ne, np.uint8) if distinct_outputs else shared["valid"][:ne]
            k = pinned(ne, np.int32) if distinct_outputs else shared["checks"][:ne]
            q1, q2 = qpool[d][off:off + ne], q2pool[d][off:off + ne]
            reqs.append(edges_request(scene_ids[s], q1, q2, v, k, step=0.05))
            keep += [v, k]
            meta.append(("edges", size, ne, s, q1, q2, v, k))
        else:
            q = qpool[d][off:off + size]
            v = pinned(size, np.uint8) if distinct_outputs else shared["valid"][:size]
            dd = None
            if kind == 1:
                dd = pinned(size, np.float64) if distinct_outputs else shared["dist"][:size]
            reqs.append(configs_request(scene_ids[s], q, v, dd))
            keep += [v, dd]
            meta.append(("valid" if kind == 0 else "distance", size, size, s, q, None, v, dd))
    return {"scene_ids": scene_ids, "scene_robot": scene_robot, "scene_n": scene_n, "robots": robots, "requests": reqs,
            "arrivals": arrivals, "meta": meta, "motions": motions, "pools": (qpool, q2pool, shared), "keep": keep,
            "scenes": sc_aabb}


def latency_summary(timings, meta, bucket=(2048, 8192)):
    """Latency percentiles; the size buckets hold the configuration and edge
    requests (the DRGBT steps are reported on their own)."""
    lat = np.array([t.t_done - t.t_submit for t in timings])
    ok = np.array([t.status == 0 for t in timings])
    sizes = np.array([m[1] for m in meta])
    checks = np.array([m[0] in ("valid", "distance", "edges") for m in meta])
    sel = ok & checks & (sizes >= bucket[0]) & (sizes <= bucket[1])
    small = ok & checks & (sizes <= 4096)
    kinds = np.array([m[0] for m in meta])
    pct = lambda a, p: float(np.percentile(a, p)) * 1e3 if a.size else None
    work = sum(m[2] for m, o in zip(meta, ok) if o)
    span = max(t.t_done for t in timings) - min(t.t_submit for t in timings) if timings else 0.0
    return {"requests": int(len(timings)), "completed": int(ok.sum()),
            "rejected": int(sum(t.status == -5 for t in timings)),
            "p50_ms": pct(lat[ok], 50), "p99_ms": pct(lat[ok], 99),
            "p50_ms_4096": pct(lat[sel], 50), "p99_ms_4096": pct(lat[sel], 99),
            "bucket_4096": list(bucket), "p99_ms_le4096": pct(lat[small], 99),
            "queries_per_s": float(ok.sum() / span) if span > 0 else None,
            "configs_or_edges_per_s": float(work / span) if span > 0 else None,
            "mean_batch": float(np.mean([t.batch_size for t in timings])) if timings else None,
            "median_queue_ms": pct(np.array([t.t_launch - t.t_submit for t in timings])[ok], 50),
            "median_run_ms": pct(np.array([t.t_done - t.t_launch for t in timings])[ok], 50),
            # the bucket by kind: "4096-config requests" are the isValid and distance
            # requests; an edge request of that many edges checks several
            # configurations per edge (and counts 8 units per edge in the classes)
            "bucket_4096_by_kind": {k: {"requests": int((sel & (kinds == k)).sum()),
                                        "p50_ms": pct(lat[sel & (kinds == k)], 50),
                                        "p99_ms": pct(lat[sel & (kinds == k)], 99)}
                                    for k in ("valid", "distance", "edges")},
            "p99_ms_4096_configs": pct(lat[sel & (kinds != "edges")], 99),
            "drgbt_horizon": {"requests": int((ok & (kinds == "reached")).sum()),
                              "p50_ms": pct(lat[ok & (kinds == "reached")], 50),
                              "p99_ms": pct(lat[ok & (kinds == "reached")], 99)},
            "motion_validity": {"requests": int((ok & (kinds == "motion")).sum()),
                                "p50_ms": pct(lat[ok & (kinds == "motion")], 50),
                                "p99_ms": pct(lat[ok & (kinds == "motion")], 99)}}
