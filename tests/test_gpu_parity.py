"""GPU parity: the CUDA forms against the oracle on the same seeded inputs.

Bars (per form):
  fp64          isValid bit-equal to ref64; distance within 1e-9 m of ref64
                (and, with the shared-bits sincos and no contraction, bit-equal)
  fp32_ref      bit-equal to ref32 (the reference's own numerics)
  fp32_recheck  isValid bit-equal to ref64 (0 flips); distance within 1e-5 m
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import robots, scenes

pytestmark = pytest.mark.gpu

DIST_TOL = {"fp64": 1e-9, "fp32_ref": 0.0, "fp32_recheck": 1e-5}
ORACLE_OF = {"fp64": "ref64", "fp32_ref": "ref32", "fp32_recheck": "ref64"}


def run_gpu(engine, robot, scene, q, prec, profile=True):
    rid = engine.upload_robot(robot)
    sid = engine.create_scene(rid, scene)
    qd = torch.from_numpy(q).cuda()
    C, L = q.shape[0], robot.num_links
    valid = torch.zeros(C, dtype=torch.uint8, device="cuda")
    dist = torch.zeros(C, dtype=torch.float64, device="cuda")
    prof = torch.zeros((C, L), dtype=torch.float32, device="cuda") if profile else None
    engine.check_configs(sid, qd, prec, valid, dist, prof)
    engine.sync()
    st = engine.stats()
    engine.destroy_scene(sid)
    return valid.cpu().numpy(), dist.cpu().numpy(), (prof.cpu().numpy() if profile else None), st


def compare(engine, robot, scene, q, prec):
    v, d, p, st = run_gpu(engine, robot, scene, q, prec)
    rv, rd, rp = O.check_configs(robot, scene, q, prec=ORACLE_OF[prec])
    flips = int((v != rv).sum())
    derr = float(np.abs(d - rd).max())
    assert flips == 0, "%s: %d isValid mismatches" % (prec, flips)
    assert derr <= DIST_TOL[prec], "%s: max distance error %g" % (prec, derr)
    if prec != "fp32_recheck":
        perr = float(np.abs(p.astype(np.float64) - rp).max())
        assert perr <= max(DIST_TOL[prec], 0.0) + (0 if prec == "fp32_ref" else 1e-7), "%s profile err %g" % (prec, perr)
    else:
        perr = float(np.abs(p.astype(np.float64) - rp).max())
        assert perr <= 2e-5, "profile err %g" % perr
    return st, derr


@pytest.mark.parametrize("prec", ["fp64", "fp32_ref", "fp32_recheck"])
def test_planar_2dof(engine, prec):
    robot, scene, q = scenes.planar_2dof_workload(65536, seed=0)
    compare(engine, robot, scene, q, prec)


@pytest.mark.parametrize("prec", ["fp64", "fp32_ref", "fp32_recheck"])
def test_xarm6(engine, prec):
    robot, scene, q = scenes.xarm6_workload(65536, seed=1)
    st, derr = compare(engine, robot, scene, q, prec)
    if prec == "fp32_recheck":
        assert st["rechecked"] < 0.5 * q.shape[0]


@pytest.mark.parametrize("workload", ["xarm6", "planar_2dof", "spatial_10dof"])
def test_order_free_kinds_and_binned_order(engine, workload):
    """isValid alone and the distance alone (no profile) in the FP32 + recheck
    form: the kernel kinds that visit links out of order with one queue across
    links and cull obstacles per warp.  A batch of 65,536 is checked in binned
    order, batches of 8,192 in index order; both give the same bits, with 0
    isValid flips and distances within 1e-5 m of ref64."""
    if workload == "xarm6":
        robot, scene, q = scenes.xarm6_workload(65536, seed=31)
    elif workload == "planar_2dof":
        robot, scene, q = scenes.planar_2dof_workload(65536, seed=32)
    else:
        rng = np.random.default_rng(33)
        robot = robots.spatial(10, radius=0.03)
        scene = scenes.random_obb_scene(rng, 30, 0.02, 0.1, scenes.SPATIAL_WS_CENTER, 1.2, rotated=True,
                                        reject_robot=robot)
        q = scenes.uniform_configs(rng, 65536, 10)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    C = q.shape[0]
    qd = torch.from_numpy(q).cuda()
    outs = {}
    engine.set_layout("lane")
    try:
        for name, step in (("binned", C), ("index_order", 8192)):
            v = torch.zeros(C, dtype=torch.uint8, device="cuda")
            d = torch.zeros(C, dtype=torch.float64, device="cuda")
            for a in range(0, C, step):
                engine.check_configs(sid, qd[a:a + step], "fp32_recheck", v[a:a + step], None, None)
                engine.check_configs(sid, qd[a:a + step], "fp32_recheck", None, d[a:a + step], None)
            engine.sync()
            outs[name] = (v.cpu().numpy(), d.cpu().numpy())
    finally:
        engine.set_layout("auto")
    engine.destroy_scene(sid)
    (vb, db), (vi, di) = outs["binned"], outs["index_order"]
    assert np.array_equal(vb, vi) and np.array_equal(db.view(np.uint64), di.view(np.uint64))
    rv, rd, _ = O.check_configs(robot, scene, q, prec="ref64", want=("valid", "dist"))
    assert int((vb != rv).sum()) == 0
    assert float(np.abs(db - rd).max()) <= 1e-5


def test_fp64_bits(engine):
    robot, scene, q = scenes.xarm6_workload(16384, seed=5)
    v, d, p, _ = run_gpu(engine, robot, scene, q, "fp64")
    rv, rd, rp = O.check_configs(robot, scene, q, prec="ref64")
    assert np.array_equal(v, rv)
    assert np.array_equal(d.view(np.uint64), rd.view(np.uint64))


def test_skeleton_fp64_bits(engine):
    robot, scene, q = scenes.xarm6_workload(4096, seed=7)
    rid = engine.upload_robot(robot)
    qd = torch.from_numpy(q).cuda()
    out = torch.zeros((q.shape[0], robot.num_links + 1, 3), dtype=torch.float64, device="cuda")
    engine.skeleton(rid, qd, out, "fp64")
    engine.sync()
    ref = O.skeleton(robot, q, prec="ref64")
    assert np.array_equal(out.cpu().numpy().view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("prec", ["fp32_recheck", "fp64"])
def test_host_buffers_pinned_and_pageable(engine, prec):
    """rpm_check_configs_host: pinned buffers (read and written by the kernels in
    host memory) and pageable ones (staged in chunks) give the device run's results."""
    import torch
    from rpmplv2_gb300 import serve
    robot, scene, q = scenes.xarm6_workload(300_000, seed=57)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    C = q.shape[0]
    v_dev = torch.zeros(C, dtype=torch.uint8, device="cuda")
    d_dev = torch.zeros(C, dtype=torch.float64, device="cuda")
    engine.check_configs(sid, torch.from_numpy(q).cuda(), prec, v_dev, d_dev, None)
    engine.sync()
    vp, dp, _ = engine.check_configs_host(sid, q, prec, want=("valid", "dist"))
    assert np.array_equal(vp, v_dev.cpu().numpy()) and np.array_equal(dp.view(np.uint64), d_dev.cpu().numpy().view(np.uint64))
    qs = serve.pinned(q.shape, np.float32)
    qs[:] = q
    vs = serve.pinned(C, np.uint8)
    ds = serve.pinned(C, np.float64)
    import ctypes
    lib = engine.lib
    from rpmplv2_gb300._abi import PRECISIONS
    assert lib.rpm_check_configs_host(engine.ctx, sid, PRECISIONS[prec], qs.ctypes.data, C, vs.ctypes.data,
                                      ds.ctypes.data, None) == 0
    assert np.array_equal(vs, v_dev.cpu().numpy()) and np.array_equal(ds.view(np.uint64), d_dev.cpu().numpy().view(np.uint64))
    engine.destroy_scene(sid)


BAND_M = 1e-5   # FP32 rounding band of a decision margin (metres over error amplification)


@pytest.mark.parametrize("prec", ["fp64", "fp32_recheck"])
def test_flips_against_reference_numerics(engine, prec):
    """Flip accounting against ref32, the reference's own FP32 numerics: the
    FP64-pinned forms may answer differently from it only where the FP64
    decision margin (rpm_decision_margins) lies inside the FP32 rounding
    band; isValid flips and distance differences above 1e-5 m are counted and
    each must have such a margin.  The reference-numerics form has none."""
    robot, scene, q = scenes.xarm6_workload(262144, seed=31)
    v, d, _, _ = run_gpu(engine, robot, scene, q, prec, profile=False)
    rv, rd, _ = O.check_configs(robot, scene, q, prec="ref32", want=("valid", "dist"))
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    C = q.shape[0]
    mv = torch.zeros(C, dtype=torch.float64, device="cuda")
    md = torch.zeros(C, dtype=torch.float64, device="cuda")
    engine.decision_margins(sid, torch.from_numpy(q).cuda(), mv, md)
    engine.sync()
    engine.destroy_scene(sid)
    mv, md = mv.cpu().numpy(), md.cpu().numpy()
    flips = np.nonzero(v != rv)[0]
    dflips = np.nonzero(np.abs(d - rd) > 1e-5)[0]
    print("%s vs ref32: %d isValid flips, %d distance differences > 1e-5 m; %d configurations inside the band"
          % (prec, flips.size, dflips.size, int((mv < BAND_M).sum())))
    assert np.all(mv[flips] < BAND_M), mv[flips]
    assert np.all(md[dflips] < BAND_M), md[dflips]
    # the band is narrow: almost every configuration is decided far from it
    assert (mv < BAND_M).sum() < 1e-3 * C


def test_reference_numerics_form_has_no_flips(engine):
    robot, scene, q = scenes.xarm6_workload(262144, seed=31)
    v, d, _, _ = run_gpu(engine, robot, scene, q, "fp32_ref", profile=False)
    rv, rd, _ = O.check_configs(robot, scene, q, prec="ref32", want=("valid", "dist"))
    assert np.array_equal(v, rv) and np.array_equal(d.view(np.uint64), rd.view(np.uint64))
