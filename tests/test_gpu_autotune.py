"""The tile-shape autotuner and its JSON cache (rpm_autotune_configs,
rpm_autotune_edges, rpm_tuning_save / rpm_tuning_load, rpm_last_shape):
tuning picks a shape per bucket, a cache written and read back drives the
launch shape of later calls, and no shape changes a result."""
import json
import os
import tempfile

import numpy as np
import pytest
import torch

from oracle import oracle as O
from rpmplv2_gb300 import scenes, serve

pytestmark = pytest.mark.gpu


def _check(engine, sid, q, dist=True):
    C = q.shape[0]
    v = torch.full((C,), 7, dtype=torch.uint8, device="cuda")
    d = torch.full((C,), -1.0, dtype=torch.float64, device="cuda") if dist else None
    engine.check_configs(sid, q, "fp32_recheck", v, d)
    engine.sync()
    return v.cpu().numpy(), (d.cpu().numpy() if dist else None), engine.last_shape()


def test_tuning_cache_drives_the_launch_shape(engine):
    rng = np.random.default_rng(61)
    robot = serve.make_robot("spatial_22dof")
    sc = serve._scene_for(robot, rng, 600)
    sid = engine.create_scene(engine.upload_robot(robot), sc)
    qh = scenes.uniform_configs(rng, 8192, 22)
    q = torch.from_numpy(qh).cuda()
    v = torch.zeros(8192, dtype=torch.uint8, device="cuda")
    d = torch.zeros(8192, dtype=torch.float64, device="cuda")
    best = engine.autotune_configs(sid, q, "fp32_recheck", v, d, reps=2)
    assert best["layout"] in ("lane", "warp") and best["ms"] > 0
    v0, d0, shape = _check(engine, sid, q)
    assert shape["layout"] == best["layout"]
    rv, rd, _ = O.check_configs(robot, sc, qh, prec="ref64", want=("valid", "dist"))
    assert np.array_equal(v0, rv) and np.abs(d0 - rd).max() <= 1e-5
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "shapes.json")
        engine.tuning_save(path)
        doc = json.load(open(path))
        assert doc["entries"] and all(e["edges"] in (0, 1) for e in doc["entries"])
        # an edited cache: the other layout, and in the warp layout 3 configurations per warp
        for e in doc["entries"]:
            if e["edges"] == 0:
                e["layout"] = 2 if best["layout"] == "lane" else 1
                e["configs_per_warp"] = 3 if e["layout"] == 2 else 0
        with open(path, "w") as f:
            f.write('{\n "entries": [\n' + ",\n".join("  " + json.dumps(e) for e in doc["entries"]) + "\n ]\n}\n")
        engine.tuning_load(path)
    v1, d1, shape1 = _check(engine, sid, q)
    assert shape1["layout"] != best["layout"]
    if shape1["layout"] == "warp":
        assert shape1["configs_per_warp"] == 3
    assert np.array_equal(v1, v0) and np.array_equal(d1.view(np.uint64), d0.view(np.uint64))
    # removing the entry returns the bucket to the built-in rule
    engine.set_tile_shape(sid, "fp32_recheck", 8192, outputs=3, layout=None)
    v2, d2, _ = _check(engine, sid, q)
    assert np.array_equal(v2, v0) and np.array_equal(d2.view(np.uint64), d0.view(np.uint64))
    engine.destroy_scene(sid)


def test_edge_shapes_set_by_hand(engine):
    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(4096, seed=62)
    sid = engine.create_scene(engine.upload_robot(robot), scene)
    q1d, q2d = torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda()
    rv, rk = O.check_edges(robot, scene, q1, q2, step=step, prec="ref64")
    for layout, g, ctas in (("lane", 0, 2), ("warp", 2, 0), ("warp", 0, 0)):
        engine.set_tile_shape(sid, "fp32_recheck", 4096, edges=True, layout=layout, configs_per_warp=g, ctas_per_sm=ctas)
        v = torch.full((4096,), 7, dtype=torch.uint8, device="cuda")
        k = torch.zeros(4096, dtype=torch.int32, device="cuda")
        engine.check_edges(sid, q1d, q2d, v, k, step=float(step), precision="fp32_recheck")
        engine.sync()
        sh = engine.last_shape()
        assert sh["layout"] == layout
        if layout == "lane":
            assert sh["ctas_per_sm"] == ctas
        elif g:
            assert sh["configs_per_warp"] == g
        assert np.array_equal(v.cpu().numpy(), rv) and np.array_equal(k.cpu().numpy(), rk)
    engine.destroy_scene(sid)
