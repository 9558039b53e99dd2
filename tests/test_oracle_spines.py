"""The oracle's bubble and spine steps (test infrastructure checks, CPU):
known radii, the spine step against a plain float32 restatement, and the
bubble's guarantee -- every configuration on the straight line from q to an
Advanced or Reached spine end is collision-free."""
import numpy as np
import pytest

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes, serve


def test_enclosing_radii_planar_known():
    """Planar2DOF at q = 0: skeleton (0,0,0), (1,0,0), (2,0,0) (Planar2DOF.cpp:132-148)."""
    rb = robots.planar_2dof(radius=0.025)
    R = O.enclosing_radii(rb, np.zeros((1, 2), np.float32))[0]
    r = np.float32(0.025)
    assert R.shape == (2, 3)
    assert R[0, 0] == 0 and R[1, 0] == 0 and R[1, 1] == 0
    assert R[0, 1] == np.float32(1) + r and R[0, 2] == np.float32(2) + r and R[1, 2] == np.float32(1) + r


def test_enclosing_radii_spatial_row0_projected():
    """Spatial10DOF at q = 0: the chain stands on the z axis, so row 0 (points
    projected on {x, y}, Spatial10DOF.cpp:17-18) is the radius alone."""
    rb = robots.spatial(10, radius=0.03)
    R = O.enclosing_radii(rb, np.zeros((1, 10), np.float32))[0]
    assert np.all(R[0, 1:] == np.float32(0.03))
    sk = O.skeleton(rb, np.zeros((1, 10), np.float32), prec="ref32")[0].astype(np.float32)
    # row 1: cumulative max of |p_j - p_1| + r
    d = [np.float32(np.linalg.norm(sk[j] - sk[1])) + np.float32(0.03) for j in range(2, 11)]
    assert np.allclose(R[1, 2:], np.maximum.accumulate(d), rtol=0, atol=1e-6)
    assert np.all(np.tril(R, 0) == 0)


def test_enclosing_radii_xarm6_structure():
    """xArm6.cpp:243-270: R(0, 1) and row 3 up to column 4 stay 0, the last row is 0,
    rows are non-decreasing."""
    rb = robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2)
    q = scenes.uniform_configs(np.random.default_rng(1), 64, 6)
    R = O.enclosing_radii(rb, q)
    assert np.all(R[:, 0, 1] == 0) and np.all(R[:, 3, :5] == 0) and np.all(R[:, 5, :] == 0)
    assert np.all(np.diff(R[:, :, 1:], axis=2) >= 0)


def _spine_py(rb, q, qe, d, prof):
    """One spine iteration (NUM_ITER_SPINE = 1) in float32 scalars, sums in index order."""
    D = rb.num_dofs
    R = O.enclosing_radii(rb, q[None])[0]
    dq = np.abs(qe - q).astype(np.float32)
    step = np.float32(np.inf)
    for i in range(D):
        s = np.float32(0)
        for k in range(D):
            s = np.float32(s + np.float32(R[k, i + 1] * dq[k]))
        with np.errstate(divide="ignore"):   # an all-zero column (xArm6 column 1): +inf, as in the reference
            v = np.float32(np.float32(prof[i] - np.float32(0)) / s)
        step = v if v < step else step
    if step > 1:
        return qe.copy(), 3
    return np.float32(q + np.float32(step) * np.float32(qe - q)).astype(np.float32), 1


def test_spine_single_iteration_matches_restatement():
    rng = np.random.default_rng(2)
    for rb in (robots.spatial(10, radius=0.03), robots.xarm6(radius=0.05, gripper_length=0.1, ground_included=2),
               robots.planar_2dof(radius=0.0)):
        D = rb.num_dofs
        q = scenes.uniform_configs(rng, 40, D)
        qe = scenes.uniform_configs(rng, 40, D)
        prof = rng.uniform(0.01, 0.5, (40, D)).astype(np.float32)
        dist = prof.min(axis=1)
        qn, st = O.extend_spines(rb, q, qe, dist, prof, num_iter=1, expanded=True)
        for c in range(40):
            want, ws = _spine_py(rb, q[c], qe[c], dist[c], prof[c])
            assert st[c] == ws
            assert np.array_equal(qn[c].view(np.uint32), want.view(np.uint32))
    # d <= 0: Trapped at q
    qn, st = O.extend_spines(rb, q[:3], qe[:3], np.zeros(3, np.float32), prof[:3])
    assert np.all(st == 2) and np.array_equal(qn, q[:3])


@pytest.mark.parametrize("name", ["spatial_10dof", "xarm6"])
def test_bubble_is_collision_free(name):
    """The bubble guarantee (RBTConnect.cpp:85-150): along the straight line from q
    to the spine's end every configuration is valid, for 1 and 5 iterations."""
    rng = np.random.default_rng(3)
    rb = serve.make_robot(name)
    scene = serve._scene_for(rb, rng, 60)
    D = rb.num_dofs
    q = scenes.uniform_configs(rng, 400, D)
    v, d, p = O.check_configs(rb, scene, q, prec="ref32")
    free = (v == 1) & (d > 0)
    q, d, p = q[free][:60], d[free][:60].astype(np.float32), p[free][:60]
    qe = scenes.uniform_configs(rng, q.shape[0], D)
    for it in (1, 5):
        qn, st = O.extend_spines(rb, q, qe, d, p, num_iter=it, expanded=True)
        assert set(np.unique(st)) <= {1, 3}
        t = np.linspace(0, 1, 33, dtype=np.float32)[:, None, None]
        path = (q[None] + t * (qn - q)[None]).reshape(-1, D).astype(np.float32)
        pv, _, _ = O.check_configs(rb, scene, path, prec="ref64", want=("valid",))
        assert pv.all()


def test_reached_states_first_layer_is_the_spine():
    """With one layer the reached state is extendSpine from the current state with
    its own distance and profile (RGBTConnect.cpp:82-85)."""
    rng = np.random.default_rng(4)
    rb = serve.make_robot("spatial_14dof")
    scene = serve._scene_for(rb, rng, 40)
    D = rb.num_dofs
    qs = scenes.uniform_configs(rng, 200, D)
    v, d, p = O.check_configs(rb, scene, qs, prec="ref32")
    c = int(np.argmax(d))
    qc = qs[c]
    hz = scenes.uniform_configs(rng, 16, D)
    q1, s1 = O.reached_states(rb, scene, qc, hz, num_layers=1, num_iter=1)
    qn, sn = O.extend_spines(rb, np.repeat(qc[None], 16, 0), hz, np.full(16, d[c], np.float32),
                             np.repeat(p[c][None], 16, 0), num_iter=1)
    assert np.array_equal(q1, qn) and np.array_equal(s1, sn)
    q5, s5 = O.reached_states(rb, scene, qc, hz, num_layers=5, num_iter=1)
    assert set(np.unique(s5)) <= {1, 3}
