"""GPU parity of the bubble and spine steps against the oracle, bit for bit
(both run the reference's float numerics): computeEnclosingRadii,
RBTConnect::extendSpine and DRGBT::computeReachedState over a horizon."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes, serve

pytestmark = pytest.mark.gpu
ROBOTS = ["planar_2dof", "xarm6", "spatial_10dof", "spatial_22dof"]


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ROBOTS)
def test_enclosing_radii(engine, name):
    rb = serve.make_robot(name)
    q = scenes.uniform_configs(np.random.default_rng(81), 3000, rb.num_dofs)
    rid = engine.upload_robot(rb)
    D = rb.num_dofs
    out = torch.zeros((q.shape[0], D, D + 1), dtype=torch.float32, device="cuda")
    engine.enclosing_radii(rid, _t(q), out)
    engine.sync()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), O.enclosing_radii(rb, q).view(np.uint32))


@pytest.mark.parametrize("name", ROBOTS)
@pytest.mark.parametrize("num_iter,expanded", [(1, True), (5, True), (5, False)])
def test_extend_spines(engine, name, num_iter, expanded):
    rng = np.random.default_rng(82)
    rb = serve.make_robot(name)
    scene = serve._scene_for(rb, rng, 50)
    D = rb.num_dofs
    q = scenes.uniform_configs(rng, 2048, D)
    _, d, p = O.check_configs(rb, scene, q, prec="ref32")
    d = d.astype(np.float32)
    qe = scenes.uniform_configs(rng, 2048, D)
    qe[:64] = q[:64]                      # zero-length spines: an all-zero bubble column
    rid = engine.upload_robot(rb)
    qn = torch.zeros((2048, D), dtype=torch.float32, device="cuda")
    st = torch.zeros(2048, dtype=torch.int32, device="cuda")
    engine.extend_spines(rid, _t(q), _t(qe), _t(d), _t(p), qn, st, num_iter=num_iter, expanded=expanded)
    engine.sync()
    rq, rs = O.extend_spines(rb, q, qe, d, p, num_iter=num_iter, expanded=expanded)
    assert np.array_equal(st.cpu().numpy(), rs)
    assert np.array_equal(qn.cpu().numpy().view(np.uint32), rq.view(np.uint32))
    assert (rs == 2).any() and (rs == 3).any()   # trapped (in collision) and reached both occur


@pytest.mark.parametrize("name,n", [("xarm6", 40), ("spatial_14dof", 300), ("planar_2dof", 6), ("spatial_22dof", 0)])
def test_reached_states(engine, name, n):
    """The DRGBT horizon in one call: reached states and statuses bit-equal to the
    oracle; their computeDistance equal to the oracle's in the exact forms."""
    rng = np.random.default_rng(83)
    rb = serve.make_robot(name)
    scene = serve._scene_for(rb, rng, n) if n else scenes.Scene(np.zeros((0, 6), np.float32))
    D = rb.num_dofs
    qs = scenes.uniform_configs(rng, 300, D)
    _, d, _ = O.check_configs(rb, scene, qs, prec="ref32", want=("dist",))
    q_cur = qs[int(np.argmax(d))]
    H = 200
    hz = scenes.uniform_configs(rng, H, D)
    sid = engine.create_scene(engine.upload_robot(rb), scene)
    rq, rs = O.reached_states(rb, scene, q_cur, hz, num_layers=5, num_iter=1, expanded=True, d_crit=0.05)
    # a long horizon (final distances by the batch check) and a short one (by
    # the one-CTA-per-state nearest-point kernel)
    for h in (H, 10):
        for prec, oprec in (("fp32_ref", "ref32"), ("fp64", "ref64")):
            qr = torch.zeros((h, D), dtype=torch.float32, device="cuda")
            st = torch.zeros(h, dtype=torch.int32, device="cuda")
            dist = torch.zeros(h, dtype=torch.float64, device="cuda")
            engine.reached_states(sid, _t(q_cur), _t(hz[:h]), qr, st, dist, precision=prec, num_layers=5,
                                  num_iter=1, expanded=True, d_crit=0.05)
            engine.sync()
            assert np.array_equal(st.cpu().numpy(), rs[:h])
            assert np.array_equal(qr.cpu().numpy().view(np.uint32), rq[:h].view(np.uint32))
            _, rd, _ = O.check_configs(rb, scene, rq[:h], prec=oprec, want=("dist",))
            assert np.array_equal(dist.cpu().numpy().view(np.uint64), rd.view(np.uint64))
    # a current state in collision: every horizon state is Trapped at q_current
    if n:
        v, _, _ = O.check_configs(rb, scene, qs, prec="ref32", want=("valid",))
        if (v == 0).any():
            qc = qs[int(np.argmin(v))]
            qr = torch.zeros((H, D), dtype=torch.float32, device="cuda")
            st = torch.zeros(H, dtype=torch.int32, device="cuda")
            engine.reached_states(sid, _t(qc), _t(hz), qr, st)
            engine.sync()
            assert np.all(st.cpu().numpy() == 2) and np.all(qr.cpu().numpy() == qc[None])
    engine.destroy_scene(sid)
