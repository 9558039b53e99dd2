"""Tile-shape autotuning over a grid of workloads, and the lane / warp layout
crossover table.

python -m rpmplv2_gb300.autotune [--out shapes.json] [--precision fp32_recheck] [--reps 3] [--crossover]

For each robot (xarm6, spatial 10- and 22-DOF), scene size, batch size and
output set (isValid; isValid + computeDistance) the library's autotuner
(rpm_autotune_configs) times every candidate tile shape and keeps the fastest
for the bucket; edge batches of the spatial 10-DOF robot are tuned the same
way (rpm_autotune_edges).  The table is written with rpm_tuning_save; a
context created with RPM_TUNING_FILE naming it, or given it with
rpm_tuning_load, launches those shapes.  With --crossover the median time of
one call in the lane and in the warp layout is printed per cell instead (one
JSON line each): the data behind the built-in layout rule.
"""
import argparse
import json
import statistics

import numpy as np


def _time(eng, fn, reps):
    import torch
    ms = []
    for it in range(reps + 2):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        if it >= 2:
            ms.append(a.elapsed_time(b))
    return statistics.median(ms)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="fp32_recheck")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default="shapes.json")
    ap.add_argument("--crossover", action="store_true", help="print lane / warp times instead of tuning")
    args = ap.parse_args()

    import torch

    from . import scenes, serve
    from .engine import Engine

    eng = Engine(0)
    rng = np.random.default_rng(5)
    sizes = (10, 20, 40, 80, 150, 300, 600, 1000) if args.crossover else (10, 40, 150, 600)
    batches = (256, 2048, 8192, 32768, 65536) if args.crossover else (256, 4096, 65536)
    for name in ("xarm6", "spatial_10dof", "spatial_22dof"):
        rb = serve.make_robot(name)
        rid = eng.upload_robot(rb)
        D = rb.num_dofs
        for n in sizes:
            sid = eng.create_scene(rid, serve._scene_for(rb, rng, n))
            for B in batches:
                q = torch.from_numpy(scenes.uniform_configs(rng, B, D)).cuda()
                v = torch.zeros(B, dtype=torch.uint8, device="cuda")
                d = torch.zeros(B, dtype=torch.float64, device="cuda")
                for kind in ("valid", "valid+dist"):
                    dd = d if kind != "valid" else None
                    if args.crossover:
                        res = {}
                        for lay in ("lane", "warp"):
                            eng.set_layout(lay)
                            res[lay] = _time(eng, lambda: eng.check_configs(sid, q, args.precision, v, dd), args.reps)
                        eng.set_layout("auto")
                        print(json.dumps({"robot": name, "n": n, "B": B, "kind": kind, **res}), flush=True)
                    else:
                        best = eng.autotune_configs(sid, q, args.precision, v, dd, reps=args.reps)
                        print(json.dumps({"robot": name, "n": n, "B": B, "kind": kind, **best}), flush=True)
            if not args.crossover and name == "spatial_10dof":
                for E in (4096, 65536):
                    q1 = scenes.uniform_configs(rng, E, D)
                    u = rng.normal(size=(E, D))
                    u /= np.linalg.norm(u, axis=1, keepdims=True)
                    q2 = (q1 + u * rng.uniform(0.01, 2.0, (E, 1))).astype(np.float32)
                    q1d, q2d = torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda()
                    ve = torch.zeros(E, dtype=torch.uint8, device="cuda")
                    best = eng.autotune_edges(sid, q1d, q2d, ve, step=0.05, precision=args.precision, reps=args.reps)
                    print(json.dumps({"robot": name, "n": n, "edges": E, **best}), flush=True)
            eng.destroy_scene(sid)
    if not args.crossover:
        eng.tuning_save(args.out)
        print("wrote", args.out)


if __name__ == "__main__":
    main()
