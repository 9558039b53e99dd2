"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.  See rpm_oracle.cpp for what it restates.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)
_u8 = ctypes.POINTER(ctypes.c_uint8)
_i32 = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_check_configs.argtypes = [_vp, _f, _f, _u8, ctypes.c_int, _f, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                        _vp, _u8, _d, _f, ctypes.c_int]
        L.orc_check_edges.argtypes = [_vp, _f, _f, _u8, ctypes.c_int, _f, _f, ctypes.c_int64, ctypes.c_float,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _u8, _i32, ctypes.c_int]
        L.orc_skeleton.argtypes = [_vp, _f, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _d]
        L.orc_sincos.argtypes = [_d, ctypes.c_int64, ctypes.c_int, _d, _d]
        L.orc_distance_nearest.argtypes = [_vp, _f, _f, _u8, ctypes.c_int, _f, ctypes.c_int64, ctypes.c_int,
                                           ctypes.c_int, _vp, _d, _f, _f, _u8]
        L.orc_prim_collision.argtypes = [_f, _f, ctypes.c_float, _f, ctypes.c_int, _vp]
        L.orc_prim_distance.argtypes = [_f, _f, ctypes.c_float, _f, ctypes.c_int, _vp, _f, ctypes.POINTER(ctypes.c_int)]
        L.orc_prim_distance.restype = ctypes.c_double
        L.orc_prim_segseg.argtypes = [_f, _f, _f, _f, ctypes.c_int, _vp]
        L.orc_prim_segseg.restype = ctypes.c_double
        L.orc_box_aabb.argtypes = [_f, _f, _f, _f]
        L.orc_undefined_hits.restype = ctypes.c_int64
        L.orc_distance_underest.argtypes = [_vp, ctypes.c_int, _f, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _vp, _f,
                                            _d, _f, _u8]
        L.orc_motion_validity.argtypes = [_vp, _f, _f, _u8, ctypes.c_int, _f, _f, ctypes.c_int64, _vp, ctypes.c_int,
                                          ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _u8, _i32]
        L.orc_enclosing_radii.argtypes = [_vp, _f, ctypes.c_int64, ctypes.c_int, _f]
        L.orc_extend_spines.argtypes = [_vp, _f, _f, _f, _f, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _f, _i32]
        L.orc_reached_states.argtypes = [_vp, _f, _f, _u8, ctypes.c_int, _f, _f, ctypes.c_int64, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, _vp, _f, _i32]
        _lib = L
    return _lib


def ref():
    """The reference's own CollisionAndDistance.cpp (None when its tree is absent)."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        R = ctypes.CDLL(path)
        R.ref_set_config.argtypes = [ctypes.c_float, ctypes.c_float]
        R.ref_collision.argtypes = [_f, _f, ctypes.c_float, _f]
        R.ref_distance.argtypes = [_f, _f, ctypes.c_float, _f, _f, ctypes.POINTER(ctypes.c_int)]
        R.ref_distance.restype = ctypes.c_float
        R.ref_segseg.argtypes = [_f, _f, _f, _f]
        R.ref_segseg.restype = ctypes.c_float
        R.ref_set_config(1e-4, 1000.0)
        _ref = R
    return _ref


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _prec(prec):
    return {"ref32": 32, "ref64": 64, 32: 32, 64: 64}[prec]


def check_configs(robot, scene, q, prec="ref64", trig=0, want=("valid", "dist", "profile"), nthreads=0):
    q = np.ascontiguousarray(q, np.float32)
    C = q.shape[0]
    L = robot.num_links
    valid = np.zeros(C, np.uint8) if "valid" in want else None
    dist = np.zeros(C, np.float64) if "dist" in want else None
    prof = np.zeros((C, L), np.float32) if "profile" in want else None
    lib().orc_check_configs(ctypes.byref(robot.desc), _p(scene.aabb, _f), _p(scene.tol, _f), _p(scene.flags, _u8),
                            scene.n, _p(q, _f), C, _prec(prec), trig, None, _p(valid, _u8), _p(dist, _d),
                            _p(prof, _f), nthreads)
    return valid, dist, prof


def check_edges(robot, scene, q1, q2, step=0.0, num_checks=10, prec="ref64", trig=0, nthreads=0):
    q1 = np.ascontiguousarray(q1, np.float32)
    q2 = np.ascontiguousarray(q2, np.float32)
    E = q1.shape[0]
    valid = np.zeros(E, np.uint8)
    checks = np.zeros(E, np.int32)
    lib().orc_check_edges(ctypes.byref(robot.desc), _p(scene.aabb, _f), _p(scene.tol, _f), _p(scene.flags, _u8),
                          scene.n, _p(q1, _f), _p(q2, _f), E, float(step), int(num_checks), _prec(prec), trig, None,
                          _p(valid, _u8), _p(checks, _i32), nthreads)
    return valid, checks


def skeleton(robot, q, prec="ref64", trig=0):
    q = np.ascontiguousarray(q, np.float32)
    C = q.shape[0]
    out = np.zeros((C, robot.num_links + 1, 3), np.float64)
    lib().orc_skeleton(ctypes.byref(robot.desc), _p(q, _f), C, _prec(prec), trig, _p(out, _d))
    return out


def distance_nearest(robot, scene, q, prec="ref64", trig=0):
    q = np.ascontiguousarray(q, np.float32)
    C, L, n = q.shape[0], robot.num_links, scene.n
    dist = np.zeros(C, np.float64)
    prof = np.zeros((C, L), np.float32)
    near = np.zeros((C, n, 6, L), np.float32)
    nv = np.zeros(C, np.uint8)
    lib().orc_distance_nearest(ctypes.byref(robot.desc), _p(scene.aabb, _f), _p(scene.tol, _f), _p(scene.flags, _u8),
                               n, _p(q, _f), C, _prec(prec), trig, None, _p(dist, _d), _p(prof, _f), _p(near, _f),
                               _p(nv, _u8))
    return dist, prof, near, nv


def distance_underestimation(robot, scene_n, q, nearest, prec="ref64", trig=0):
    """computeDistanceUnderestimation from nearest points (C x n x 6 x L float32).
    Returns (dist, profile, complete)."""
    q = np.ascontiguousarray(q, np.float32)
    nearest = np.ascontiguousarray(nearest, np.float32)
    C, L = q.shape[0], robot.num_links
    dist = np.zeros(C, np.float64)
    prof = np.zeros((C, L), np.float32)
    comp = np.zeros(C, np.uint8)
    lib().orc_distance_underest(ctypes.byref(robot.desc), int(scene_n), _p(q, _f), C, _prec(prec), trig, None,
                                _p(nearest, _f), _p(dist, _d), _p(prof, _f), _p(comp, _u8))
    return dist, prof, comp


def enclosing_radii(robot, q, trig=0):
    """computeEnclosingRadii per configuration: (C, D, D + 1) float32."""
    q = np.ascontiguousarray(q, np.float32)
    C, D = q.shape
    out = np.zeros((C, D, D + 1), np.float32)
    lib().orc_enclosing_radii(ctypes.byref(robot.desc), _p(q, _f), C, trig, _p(out, _f))
    return out


def extend_spines(robot, q, qe, dist, profile, num_iter=1, expanded=True, trig=0):
    """RBTConnect::extendSpine per row; dist (C,) and profile (C, L) float32.
    Returns (q_new (C, D) float32, status (C,) int32)."""
    q = np.ascontiguousarray(q, np.float32)
    qe = np.ascontiguousarray(qe, np.float32)
    dist = np.ascontiguousarray(dist, np.float32)
    profile = np.ascontiguousarray(profile, np.float32)
    C, D = q.shape
    q_new = np.zeros((C, D), np.float32)
    status = np.zeros(C, np.int32)
    lib().orc_extend_spines(ctypes.byref(robot.desc), _p(q, _f), _p(qe, _f), _p(dist, _f), _p(profile, _f), C,
                            int(num_iter), int(bool(expanded)), trig, _p(q_new, _f), _p(status, _i32))
    return q_new, status


def reached_states(robot, scene, q_cur, horizon, num_layers=5, num_iter=1, expanded=True, d_crit=0.05, trig=0):
    """DRGBT::computeReachedState for every horizon state (without the final
    computeDistance).  Returns (q_reached (H, D) float32, status (H,) int32)."""
    q_cur = np.ascontiguousarray(q_cur, np.float32).reshape(-1)
    horizon = np.ascontiguousarray(horizon, np.float32)
    H, D = horizon.shape
    q_out = np.zeros((H, D), np.float32)
    status = np.zeros(H, np.int32)
    lib().orc_reached_states(ctypes.byref(robot.desc), _p(scene.aabb, _f), _p(scene.tol, _f), _p(scene.flags, _u8),
                             scene.n, _p(q_cur, _f), _p(horizon, _f), H, int(num_layers), int(num_iter),
                             int(bool(expanded)), float(d_crit), trig, None, _p(q_out, _f), _p(status, _i32))
    return q_out, status


def motion_validity(robot, scene, q_prev, q_cur, movers, max_iter_time, num_points, prec="ref32", trig=0):
    """MotionValidity::check per motion with the boxes 'movers' (a ctypes array
    of rpm_moving_box) moving straight.  Returns (valid (M,) uint8, checks (M,) int32)."""
    q_prev = np.ascontiguousarray(q_prev, np.float32)
    q_cur = np.ascontiguousarray(q_cur, np.float32)
    M = q_prev.shape[0]
    valid = np.zeros(M, np.uint8)
    checks = np.zeros(M, np.int32)
    lib().orc_motion_validity(ctypes.byref(robot.desc), _p(scene.aabb, _f), _p(scene.tol, _f), _p(scene.flags, _u8),
                              scene.n, _p(q_prev, _f), _p(q_cur, _f), M, ctypes.addressof(movers) if len(movers) else None,
                              len(movers), float(max_iter_time), int(num_points), _prec(prec), trig, None,
                              _p(valid, _u8), _p(checks, _i32))
    return valid, checks


def sincos(x, trig=0):
    x = np.ascontiguousarray(x, np.float64)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    lib().orc_sincos(_p(x, _d), x.size, trig, _p(s, _d), _p(c, _d))
    return s, c


def prim_collision(A, B, r, obs, prec="ref32"):
    A, B, obs = (np.ascontiguousarray(v, np.float32) for v in (A, B, obs))
    return lib().orc_prim_collision(_p(A, _f), _p(B, _f), float(r), _p(obs, _f), _prec(prec), None)


def prim_distance(A, B, r, obs, prec="ref32"):
    A, B, obs = (np.ascontiguousarray(v, np.float32) for v in (A, B, obs))
    pts = np.zeros(6, np.float32)
    hp = ctypes.c_int()
    d = lib().orc_prim_distance(_p(A, _f), _p(B, _f), float(r), _p(obs, _f), _prec(prec), None, _p(pts, _f),
                                ctypes.byref(hp))
    return d, pts, bool(hp.value)


def undefined_hits():
    """Evaluations on this thread that reached the reference's uninitialised
    edge matrix (getLineSegments selecting no edge) since the last call."""
    return int(lib().orc_undefined_hits())


def box_aabb(dim, pos, quat_xyzw):
    dim, pos, quat = (np.ascontiguousarray(v, np.float32) for v in (dim, pos, quat_xyzw))
    out = np.zeros(6, np.float32)
    lib().orc_box_aabb(_p(dim, _f), _p(pos, _f), _p(quat, _f), _p(out, _f))
    return out
