"""The oracle's MotionValidity::check with moving boxes (CPU): a known answer,
and with no motion the checks equal isValid on the interpolated points."""
import numpy as np

from oracle import oracle as O
from rpmplv2_gb300 import _abi, robots, scenes, serve


def movers_of(specs, quats=None):
    """A ctypes array of rpm_moving_box from (index, max_vel, dim, pos) tuples."""
    arr = (_abi.MovingBox * len(specs))()
    for k, (idx, v, dim, pos) in enumerate(specs):
        quat = quats[k] if quats is not None else (0.0, 0.0, 0.0, 1.0)
        arr[k] = _abi.MovingBox(idx, v, tuple(dim), tuple(pos), tuple(quat))
    return arr


def test_box_sweeping_into_a_planar_arm():
    """planar_2dof at q = 0 spans x in [0, 2]; a 0.1 m box starts at x = 3 and moves
    -x at 40 m/s; with max_iter_time 0.05 s and 10 checks each step is 0.2 m, so
    the first collision is check 5 (Environment.cpp:220-233, MotionValidity.cpp:30-53)."""
    rb = robots.planar_2dof(radius=0.0)
    box = scenes.box_aabb([0.1, 0.1, 0.1], [3.0, 0.0, 0.0])
    scene = scenes.Scene(box[None], flags=np.array([_abi.RPM_OBS_DYNAMIC], np.uint8))
    q = np.zeros((1, 2), np.float32)
    mv = movers_of([(0, 40.0, (0.1, 0.1, 0.1), (3.0, 0.0, 0.0))])
    for prec in ("ref32", "ref64"):
        v, k = O.motion_validity(rb, scene, q, q, mv, 0.05, 10, prec=prec)
        assert v[0] == 0 and k[0] == 5
    still = movers_of([(0, 0.0, (0.1, 0.1, 0.1), (3.0, 0.0, 0.0))])
    v, k = O.motion_validity(rb, scene, q, q, still, 0.05, 10)
    assert v[0] == 1 and k[0] == 10


def test_static_motion_equals_interpolated_checks():
    rng = np.random.default_rng(91)
    rb = serve.make_robot("spatial_10dof")
    scene = serve._scene_for(rb, rng, 80)
    D = rb.num_dofs
    q1 = scenes.uniform_configs(rng, 50, D)
    q2 = (q1 + rng.uniform(-0.5, 0.5, q1.shape)).astype(np.float32)
    N = 7
    v, k = O.motion_validity(rb, scene, q1, q2, movers_of([]), 0.05, N, prec="ref32")
    for m in range(50):
        a, b = q1[m], q2[m]
        ss = np.float32(0)
        for i in range(D):
            d = np.float32(a[i] - b[i])
            ss = np.float32(ss + np.float32(d * d))
        dist = np.float32(np.sqrt(ss))
        pts = []
        for kk in range(1, N + 1):
            step = np.float32(np.float32(dist * np.float32(kk)) / np.float32(N))
            r = np.float32(step / dist)
            pts.append((a + (b - a) * r).astype(np.float32))
        pv, _, _ = O.check_configs(rb, scene, np.array(pts), prec="ref32", want=("valid",))
        bad = np.nonzero(pv == 0)[0]
        assert v[m] == (1 if bad.size == 0 else 0)
        assert k[m] == (N if bad.size == 0 else bad[0] + 1)
