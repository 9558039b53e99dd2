"""Time both layouts of the configuration checks on this GPU.

python -m rpmplv2_gb300.layout_sweep [--precision fp32_recheck] [--reps 5]

For each robot (xarm6, spatial 10- and 22-DOF), scene size (10-300
obstacles), batch size (256-32,768 configurations) and output set (isValid;
isValid + computeDistance), prints one JSON line with the median CUDA-event
time of one rpm_check_configs call in the lane and in the warp layout.  The
automatic layout's thresholds (kWide* in rpm_wide.cuh) are the crossovers of
this table.
"""
import argparse
import json
import statistics

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="fp32_recheck")
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()

    import torch

    from . import scenes, serve
    from .engine import Engine

    eng = Engine(0)
    rng = np.random.default_rng(5)
    for name in ("xarm6", "spatial_10dof", "spatial_22dof"):
        rb = serve.make_robot(name)
        rid = eng.upload_robot(rb)
        D = rb.num_dofs
        for n in (10, 20, 40, 80, 150, 300):
            sid = eng.create_scene(rid, serve._scene_for(rb, rng, n))
            for B in (256, 2048, 8192, 32768):
                q = torch.from_numpy(scenes.uniform_configs(rng, B, D)).cuda()
                v = torch.zeros(B, dtype=torch.uint8, device="cuda")
                d = torch.zeros(B, dtype=torch.float64, device="cuda")
                for kind in ("valid", "valid+dist"):
                    res = {}
                    for lay in ("lane", "warp"):
                        eng.set_layout(lay)
                        ms = []
                        for it in range(args.reps + 2):
                            a = torch.cuda.Event(enable_timing=True)
                            b = torch.cuda.Event(enable_timing=True)
                            a.record()
                            eng.check_configs(sid, q, args.precision, v, d if kind != "valid" else None)
                            b.record()
                            b.synchronize()
                            if it >= 2:
                                ms.append(a.elapsed_time(b))
                        res[lay] = statistics.median(ms)
                    print(json.dumps({"robot": name, "n": n, "B": B, "kind": kind, **res}), flush=True)
            eng.destroy_scene(sid)
    eng.set_layout("auto")


if __name__ == "__main__":
    main()
