"""ctypes binding of librpm_gb300.so (include/rpm_gpu.h).

There is no CPU fallback: constructing an Engine without the CUDA library or
without a GPU raises.
"""
import ctypes
import os

import numpy as np

from . import _abi
from ._abi import BatchItem, CheckStats, EdgeBatchItem, LAYOUTS, MovingBox, Params, PRECISIONS, SpineParams, TileShape

_LIB = None

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_pi32 = ctypes.POINTER(ctypes.c_int32)


class RpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rpm error %d: %s" % (code, msg))
        self.code = code


def lib_path():
    from . import build as _b
    return _b.LIB


def load(build_if_missing=False):
    """Load the CUDA library (building it first if asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("librpm_gb300.so is not built; run __graft_entry__.build() (no CPU fallback)")
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(path)
    L.rpm_last_error_string.restype = ctypes.c_char_p
    L.rpm_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(_vp)]
    L.rpm_ctx_destroy.argtypes = [_vp]
    L.rpm_ctx_set_params.argtypes = [_vp, ctypes.POINTER(Params)]
    L.rpm_robot_upload.argtypes = [_vp, ctypes.c_void_p, _pi32]
    L.rpm_scene_create.argtypes = [_vp, _i32, _vp, _vp, _vp, _i32, _pi32]
    L.rpm_scene_update.argtypes = [_vp, _i32, _vp, _vp, _i32, ctypes.POINTER(ctypes.c_uint64)]
    L.rpm_scene_destroy.argtypes = [_vp, _i32]
    L.rpm_scene_update_many.argtypes = [_vp, _i32, _vp, _vp, _vp, _vp, _vp]
    L.rpm_scene_info.argtypes = [_vp, _i32, _pi32, _pi32, ctypes.POINTER(ctypes.c_uint64)]
    L.rpm_box_aabb.argtypes = [_vp, _vp, _vp, _vp]
    L.rpm_check_configs.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp, _vp, _vp]
    L.rpm_check_batch.argtypes = [_vp, _i32, _vp, _i32, _vp]
    L.rpm_check_edges.argtypes = [_vp, _i32, _i32, _vp, _vp, _i64, ctypes.c_float, _i32, _vp, _vp, _vp]
    L.rpm_check_edges_batch.argtypes = [_vp, _i32, _vp, _i32, _vp]
    L.rpm_ctx_set_graphs.argtypes = [_vp, ctypes.c_int]
    L.rpm_ctx_set_layout.argtypes = [_vp, ctypes.c_int32]
    L.rpm_distance_nearest.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp]
    L.rpm_distance_underestimation.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp]
    L.rpm_scenario_read.argtypes = [ctypes.c_char_p, _vp, _vp, _vp, _vp, _i32]
    L.rpm_random_scenario_read.argtypes = [ctypes.c_char_p, _i32, _i32, _i32, _vp, _vp, _vp, _vp]
    L.rpm_scene_move_straight.argtypes = [_vp, _i32, _vp, _i32, ctypes.c_float, _i32, ctypes.POINTER(ctypes.c_uint64)]
    L.rpm_motion_validity.argtypes = [_vp, _i32, _i32, _vp, _vp, _i64, _vp, _i32, ctypes.c_float, _i32, _vp, _vp, _vp]
    L.rpm_enclosing_radii.argtypes = [_vp, _i32, _vp, _i64, _vp, _vp]
    L.rpm_extend_spines.argtypes = [_vp, _i32, _vp, _vp, _vp, _vp, _i64, _i32, _i32, _vp, _vp, _vp]
    L.rpm_reached_states.argtypes = [_vp, _i32, _i32, _vp, _vp, _i64, ctypes.POINTER(SpineParams), _vp, _vp, _vp, _vp]
    L.rpm_autotune_edges.argtypes = [_vp, _i32, _i32, _vp, _vp, _i64, ctypes.c_float, _i32, _vp, _i32,
                                     ctypes.POINTER(TileShape)]
    L.rpm_autotune_configs.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp, _vp, _i32, ctypes.POINTER(TileShape)]
    L.rpm_set_tile_shape.argtypes = [_vp, _i32, _i32, _i32, _i64, _i32, _vp]
    L.rpm_tuning_save.argtypes = [_vp, ctypes.c_char_p]
    L.rpm_tuning_load.argtypes = [_vp, ctypes.c_char_p]
    L.rpm_last_shape.argtypes = [_vp, _vp, ctypes.POINTER(TileShape)]
    L.rpm_check_configs_host.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp, _vp]
    L.rpm_skeleton.argtypes = [_vp, _i32, _i32, _vp, _i64, _vp, _vp]
    L.rpm_last_stats.argtypes = [_vp, _vp, ctypes.POINTER(CheckStats)]
    L.rpm_sync.argtypes = [_vp, _vp]
    L.rpm_ctx_set_timing.argtypes = [_vp, ctypes.c_int]
    L.rpm_last_timing.argtypes = [_vp, _vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.rpm_probe_fp32_peak.argtypes = [_vp, ctypes.POINTER(ctypes.c_double)]
    L.rpm_probe_bounded_wait.argtypes = [_vp, ctypes.c_uint32]
    L.rpm_robot_builtin.argtypes = [ctypes.c_char_p, _vp]
    L.rpm_decision_margins.argtypes = [_vp, _i32, _vp, _i64, _vp, _vp, _vp]
    L.rpm_probe_primitives.argtypes = [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp]
    L.rpm_check_configs_noalloc.argtypes = [_vp, _vp, _vp, _vp, _i32, ctypes.POINTER(Params), _vp, _i64, _vp, _vp,
                                            _vp, _vp]
    _LIB = L
    return L


def _check(rc):
    if rc != 0:
        raise RpmError(rc, _LIB.rpm_last_error_string().decode())


def _ptr(x):
    """Device pointer of a torch tensor, host pointer of a numpy array, or None."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


class Engine:
    """A device context: robots and scenes resident in HBM."""

    def __init__(self, device=0, equality_threshold=1e-4, max_distance=1000.0):
        self.lib = load()
        self.ctx = _vp()
        _check(self.lib.rpm_ctx_create(int(device), ctypes.byref(self.ctx)))
        self.device = device
        self.set_params(equality_threshold, max_distance)
        self._robots = {}
        self._scene_robot = {}

    def close(self):
        if self.ctx:
            self.lib.rpm_ctx_destroy(self.ctx)
            self.ctx = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, equality_threshold=1e-4, max_distance=1000.0):
        p = Params(equality_threshold, max_distance)
        _check(self.lib.rpm_ctx_set_params(self.ctx, ctypes.byref(p)))

    def upload_robot(self, robot):
        rid = _i32()
        _check(self.lib.rpm_robot_upload(self.ctx, ctypes.addressof(robot.desc), ctypes.byref(rid)))
        self._robots[rid.value] = robot
        return rid.value

    def create_scene(self, robot_id, scene):
        sid = _i32()
        _check(self.lib.rpm_scene_create(self.ctx, robot_id, scene.aabb.ctypes.data, scene.tol.ctypes.data,
                                         scene.flags.ctypes.data, scene.n, ctypes.byref(sid)))
        self._scene_robot[sid.value] = robot_id
        return sid.value

    def update_scene(self, scene_id, idx, aabb):
        idx = np.ascontiguousarray(idx, np.int32)
        aabb = np.ascontiguousarray(aabb, np.float32).reshape(-1, 6)
        ver = ctypes.c_uint64()
        _check(self.lib.rpm_scene_update(self.ctx, scene_id, idx.ctypes.data, aabb.ctypes.data, idx.size,
                                         ctypes.byref(ver)))
        return ver.value

    def update_scenes(self, updates):
        """rpm_scene_update_many: updates is a list of (scene_id, idx, aabb);
        returns the new versions."""
        sids = np.array([u[0] for u in updates], np.int32)
        counts = np.array([len(u[1]) for u in updates], np.int32)
        idx = np.ascontiguousarray(np.concatenate([np.asarray(u[1], np.int32) for u in updates]) if updates else
                                   np.zeros(0, np.int32), np.int32)
        aabb = np.ascontiguousarray(np.concatenate([np.asarray(u[2], np.float32).reshape(-1, 6) for u in updates])
                                    if updates else np.zeros((0, 6), np.float32), np.float32)
        ver = np.zeros(len(updates), np.uint64)
        _check(self.lib.rpm_scene_update_many(self.ctx, len(updates), sids.ctypes.data, counts.ctypes.data,
                                              idx.ctypes.data, aabb.ctypes.data, ver.ctypes.data))
        return [int(v) for v in ver]

    def destroy_scene(self, scene_id):
        _check(self.lib.rpm_scene_destroy(self.ctx, scene_id))

    def robot_of(self, scene_id):
        return self._robots[self._scene_robot[scene_id]]

    # ---- device-buffer calls (torch CUDA tensors) ----
    def check_configs(self, scene_id, q, precision="fp64", valid=None, dist=None, profile=None, stream=None):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        n = int(q.shape[0])
        _check(self.lib.rpm_check_configs(self.ctx, scene_id, prec, _ptr(q), n, _ptr(valid), _ptr(dist),
                                          _ptr(profile), stream))

    def check_batch(self, items, precision="fp64", stream=None):
        """items: list of (scene_id, q, valid, dist, profile) with torch CUDA tensors (outputs nullable)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        arr = (BatchItem * len(items))()
        for k, (sid, q, valid, dist, profile) in enumerate(items):
            arr[k] = BatchItem(sid, 0, _ptr(q), int(q.shape[0]), _ptr(valid), _ptr(dist), _ptr(profile))
        _check(self.lib.rpm_check_batch(self.ctx, prec, ctypes.addressof(arr), len(items), stream))

    def check_edges(self, scene_id, q1, q2, valid, checks=None, step=0.0, num_checks=10, precision="fp64",
                    stream=None):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_check_edges(self.ctx, scene_id, prec, _ptr(q1), _ptr(q2), int(q1.shape[0]), float(step),
                                        int(num_checks), _ptr(valid), _ptr(checks), stream))

    def check_edges_batch(self, items, precision="fp64", stream=None):
        """items: list of (scene_id, q1, q2, valid, checks, step, num_checks) with torch CUDA tensors
        (checks nullable); every item's edges go through one pipeline."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        arr = (EdgeBatchItem * max(1, len(items)))()
        for k, (sid, q1, q2, valid, checks, step, num_checks) in enumerate(items):
            arr[k] = EdgeBatchItem(sid, int(num_checks), int(q1.shape[0]), _ptr(q1), _ptr(q2), float(step), _ptr(valid),
                                   _ptr(checks))
        _check(self.lib.rpm_check_edges_batch(self.ctx, prec, ctypes.addressof(arr), len(items), stream))

    def motion_validity(self, scene_id, q_prev, q_cur, movers, max_iter_time, num_points, valid, checks=None,
                        precision="fp32_ref", stream=None):
        """MotionValidity::check per motion (torch CUDA tensors q_prev, q_cur [M][D], valid [M] uint8,
        checks [M] int32); movers: a ctypes array of MovingBox."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_motion_validity(self.ctx, scene_id, prec, _ptr(q_prev), _ptr(q_cur), int(q_prev.shape[0]),
                                            ctypes.addressof(movers) if len(movers) else None, len(movers),
                                            float(max_iter_time), int(num_points), _ptr(valid), _ptr(checks), stream))

    def move_straight(self, scene_id, movers, delta_time, steps):
        """Environment::moveStraight 'steps' times on the movers (positions advanced in place) and the
        device scene; returns the scene's new version."""
        ver = ctypes.c_uint64()
        _check(self.lib.rpm_scene_move_straight(self.ctx, scene_id, ctypes.addressof(movers) if len(movers) else None,
                                                len(movers), float(delta_time), int(steps), ctypes.byref(ver)))
        return ver.value

    def enclosing_radii(self, robot_id, q, radii, stream=None):
        """computeEnclosingRadii: q [C][D] float32, radii [C][D][D+1] float32 (torch CUDA tensors)."""
        _check(self.lib.rpm_enclosing_radii(self.ctx, robot_id, _ptr(q), int(q.shape[0]), _ptr(radii), stream))

    def extend_spines(self, robot_id, q, qe, dist, profile, q_new, status, num_iter=1, expanded=True, stream=None):
        """extendSpine per row (torch CUDA tensors: dist [C] float32, profile [C][L], status [C] int32)."""
        _check(self.lib.rpm_extend_spines(self.ctx, robot_id, _ptr(q), _ptr(qe), _ptr(dist), _ptr(profile),
                                          int(q.shape[0]), int(num_iter), int(bool(expanded)), _ptr(q_new),
                                          _ptr(status), stream))

    def reached_states(self, scene_id, q_current, horizon, q_reached, status, dist=None, precision="fp32_recheck",
                       num_layers=5, num_iter=1, expanded=True, d_crit=0.05, stream=None):
        """DRGBT computeReachedState for a horizon [H][D] from q_current [D] (torch CUDA tensors)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        sp = SpineParams(int(num_layers), int(num_iter), int(bool(expanded)), float(d_crit))
        _check(self.lib.rpm_reached_states(self.ctx, scene_id, prec, _ptr(q_current), _ptr(horizon),
                                           int(horizon.shape[0]), ctypes.byref(sp), _ptr(q_reached), _ptr(status),
                                           _ptr(dist), stream))

    def set_graphs(self, enable=True):
        _check(self.lib.rpm_ctx_set_graphs(self.ctx, 1 if enable else 0))

    def distance_nearest(self, scene_id, q, dist, profile, nearest, nearest_valid, precision="fp64", stream=None):
        """computeDistance with nearest points (torch CUDA tensors: q [C][D] float32, dist [C] float64,
        profile [C][L] float32, nearest [C][n][6][L] float32, nearest_valid [C] uint8)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_distance_nearest(self.ctx, scene_id, prec, _ptr(q), int(q.shape[0]), _ptr(dist),
                                             _ptr(profile), _ptr(nearest), _ptr(nearest_valid), stream))

    def distance_underestimation(self, scene_id, q, nearest, dist, profile, complete, precision="fp64", stream=None):
        """computeDistanceUnderestimation from nearest points ([C][n][6][L] float32)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_distance_underestimation(self.ctx, scene_id, prec, _ptr(q), int(q.shape[0]), _ptr(nearest),
                                                     _ptr(dist), _ptr(profile), _ptr(complete), stream))

    def set_layout(self, layout="auto"):
        """Spread configuration checks one lane ('lane') or one warp ('warp')
        per configuration, or choose per segment ('auto').  Outputs do not
        depend on it."""
        code = LAYOUTS[layout] if isinstance(layout, str) else int(layout)
        _check(self.lib.rpm_ctx_set_layout(self.ctx, code))

    def autotune_edges(self, scene_id, q1, q2, valid, step=0.0, num_checks=10, precision="fp32_recheck", reps=3):
        """rpm_autotune_edges: the fastest tile shape of this batch's bucket
        (kept in the context's table), as a dict."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        out = TileShape()
        _check(self.lib.rpm_autotune_edges(self.ctx, scene_id, prec, _ptr(q1), _ptr(q2), int(q1.shape[0]),
                                           float(step), int(num_checks), _ptr(valid), int(reps), ctypes.byref(out)))
        return out.as_dict()

    def autotune_configs(self, scene_id, q, precision="fp32_recheck", valid=None, dist=None, profile=None, reps=3):
        """rpm_autotune_configs: the fastest tile shape of this batch's bucket, as a dict."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        out = TileShape()
        _check(self.lib.rpm_autotune_configs(self.ctx, scene_id, prec, _ptr(q), int(q.shape[0]), _ptr(valid),
                                             _ptr(dist), _ptr(profile), int(reps), ctypes.byref(out)))
        return out.as_dict()

    def set_tile_shape(self, scene_id, precision, count, outputs=1, edges=False, layout=None, configs_per_warp=0,
                       ctas_per_sm=0):
        """rpm_set_tile_shape; layout None removes the bucket's entry."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        sh = None
        if layout is not None:
            sh = TileShape(LAYOUTS[layout] if isinstance(layout, str) else int(layout), int(configs_per_warp),
                           int(ctas_per_sm), 0.0)
        _check(self.lib.rpm_set_tile_shape(self.ctx, scene_id, prec, 1 if edges else 0, int(count), int(outputs),
                                           ctypes.byref(sh) if sh is not None else None))

    def tuning_save(self, path):
        _check(self.lib.rpm_tuning_save(self.ctx, str(path).encode()))

    def tuning_load(self, path):
        _check(self.lib.rpm_tuning_load(self.ctx, str(path).encode()))

    def last_shape(self, stream=None):
        out = TileShape()
        _check(self.lib.rpm_last_shape(self.ctx, stream, ctypes.byref(out)))
        return out.as_dict()

    def skeleton(self, robot_id, q, points, precision="fp64", stream=None):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_skeleton(self.ctx, robot_id, prec, _ptr(q), int(q.shape[0]), _ptr(points), stream))

    def stats(self, stream=None):
        s = CheckStats()
        _check(self.lib.rpm_last_stats(self.ctx, stream, ctypes.byref(s)))
        return {"configs": s.configs, "rechecked": s.rechecked, "overflow": s.overflow,
                "device_status": s.device_status}

    def set_timing(self, enable=True):
        _check(self.lib.rpm_ctx_set_timing(self.ctx, 1 if enable else 0))

    def last_timing(self, stream=None):
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(self.lib.rpm_last_timing(self.ctx, stream, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def fp32_peak_tflops(self):
        t = ctypes.c_double()
        _check(self.lib.rpm_probe_fp32_peak(self.ctx, ctypes.byref(t)))
        return t.value

    def sync(self, stream=None):
        _check(self.lib.rpm_sync(self.ctx, stream))

    def decision_margins(self, scene_id, q, margin_valid, margin_dist, stream=None):
        """FP64 decision margins per configuration (device tensors; see rpm_decision_margins)."""
        _check(self.lib.rpm_decision_margins(self.ctx, scene_id, _ptr(q), int(q.shape[0]), _ptr(margin_valid),
                                             _ptr(margin_dist), stream))

    def probe_primitives(self, precision, kind, a, b, x, r, value, settled=None, stream=None):
        """The device trees on single primitives (device tensors; see
        rpm_probe_primitives): kind int32 (n,), a/b float32 (n, 3), x float32
        (n, 6), r float32 (n,), value float64 (n,), settled uint8 (n,)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _check(self.lib.rpm_probe_primitives(self.ctx, prec, _ptr(kind), _ptr(a), _ptr(b), _ptr(x), _ptr(r),
                                             int(kind.shape[0]), _ptr(value), _ptr(settled), stream))

    # ---- host-buffer call (numpy) ----
    def check_configs_host(self, scene_id, q, precision="fp64", want=("valid", "dist")):
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        q = np.ascontiguousarray(q, np.float32)
        C = q.shape[0]
        L = self.robot_of(scene_id).num_links
        valid = np.zeros(C, np.uint8) if "valid" in want else None
        dist = np.zeros(C, np.float64) if "dist" in want else None
        prof = np.zeros((C, L), np.float32) if "profile" in want else None
        _check(self.lib.rpm_check_configs_host(self.ctx, scene_id, prec, q.ctypes.data, C, _ptr(valid), _ptr(dist),
                                               _ptr(prof)))
        return valid, dist, prof


def box_aabb(dim, pos, quat_xyzw=(0.0, 0.0, 0.0, 1.0)):
    L = load()
    dim, pos, quat = (np.ascontiguousarray(v, np.float32) for v in (dim, pos, quat_xyzw))
    out = np.zeros(6, np.float32)
    _check(L.rpm_box_aabb(dim.ctypes.data, pos.ctypes.data, quat.ctypes.data, out.ctypes.data))
    return out


ABI_SYMBOLS = [
    "rpm_last_error_string", "rpm_version", "rpm_ctx_create", "rpm_ctx_destroy", "rpm_ctx_set_params",
    "rpm_robot_upload", "rpm_scene_create", "rpm_scene_update", "rpm_scene_update_many", "rpm_scene_destroy", "rpm_scene_info",
    "rpm_box_aabb", "rpm_check_configs", "rpm_check_configs_host", "rpm_skeleton", "rpm_last_stats", "rpm_sync",
    "rpm_ctx_set_timing", "rpm_last_timing", "rpm_probe_fp32_peak", "rpm_probe_bounded_wait", "rpm_probe_primitives", "rpm_decision_margins", "rpm_robot_builtin", "rpm_check_configs_noalloc", "rpm_check_batch",
    "rpm_check_edges", "rpm_check_edges_batch", "rpm_ctx_set_graphs", "rpm_autotune_edges", "rpm_autotune_configs", "rpm_set_tile_shape",
    "rpm_tuning_save", "rpm_tuning_load", "rpm_last_shape", "rpm_ctx_set_layout",
    "rpm_distance_nearest", "rpm_distance_underestimation", "rpm_enclosing_radii", "rpm_extend_spines",
    "rpm_reached_states", "rpm_motion_validity", "rpm_scene_move_straight", "rpm_scenario_read", "rpm_random_scenario_read",
    "rpm_server_create", "rpm_server_submit", "rpm_server_poll", "rpm_server_wait", "rpm_server_release",
    "rpm_server_replay", "rpm_server_stats", "rpm_server_destroy",
]
