#!/usr/bin/env python
"""Benchmark of the RealVectorSpace collision + distance path on GB300.

Headline workload (one "step" = one pass over the batch): xarm6 capsule model
(radius 0.05 m, gripper 0.1 m, ground from link 2) against 50 cubes of 0.05 m
plus the ground box, 1,048,576 configurations uniform in [-pi, pi]^6; outputs
per configuration are isValid and computeDistance.

  value    configs/s of the FP32 + FP64-recheck form, inputs resident in HBM
  e2e      the same through rpm_check_configs_host with pinned host buffers
           (host->device copy of q and device->host copy of both outputs timed)
  fp64     configs/s of the plain FP64 form on the same batch, with the number
           of isValid flips and the max distance difference between the forms

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

# separate hardware queues for the serving loop's streams (before any CUDA context exists)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "xarm6 configs/s FP32+recheck vs FP64 GPU (0 flips); p50/p99 serve latency"
NUM_CONFIGS = 1 << 20
D = 6
PAIRS = 6 * 50 + 4                       # link x obstacle pairs not skipped by the ground rule
FLOP_PER_CONFIG = 60 * D + 100 * PAIRS   # fixed work convention: 30,760 FLOP per configuration
BYTES_PER_CONFIG = 4 * D + 1 + 8         # q in, isValid + distance out
WORKLOAD = ("xarm6 capsules (r 0.05 m, gripper 0.1 m, ground from link 2) vs 50 cubes of 0.05 m + ground, "
            "1,048,576 configs in [-pi, pi]^6; isValid + computeDistance")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--configs", type=int, default=NUM_CONFIGS)
    ap.add_argument("--no-extra", action="store_true", help="skip the edge, mixed-DOF, large-scene and serving measurements")
    ap.add_argument("--extra", default="planar,edges,mixed,large,serve,planner",
                    help="comma list of extra measurements: planar, edges, mixed, large, serve, planner")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms from just
    before the warm-up steps to the end of the timed region (the sampler is
    running, with a first sample taken, before the first step)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples (the JSON line carries their summary)
        self.path = os.environ.get("RPM_CLOCKS_CSV", os.path.join(tempfile.gettempdir(), "rpm_clocks_bench.csv"))

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 3.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names[1:], p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(robot, scene, q, sample):
    """The oracle (a restatement of the reference's FP32 path) on every host
    core.  Returns the baseline line and the oracle's outputs (ref32 valid,
    distance) on the sample, which the parity accounting then uses."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    qs = np.ascontiguousarray(q[:sample])
    O.check_configs(robot, scene, qs[:4096], prec="ref32", nthreads=cores)   # warm-up
    t0 = time.perf_counter()
    rv, rd, _ = O.check_configs(robot, scene, qs, prec="ref32", nthreads=cores)
    dt = time.perf_counter() - t0
    t1 = time.perf_counter()
    O.check_configs(robot, scene, qs[:65536], prec="ref32", nthreads=1)
    dt1 = time.perf_counter() - t1
    line = {"value": sample / dt, "unit": "configs/s", "cores": cores, "kind": "port",
            "sample": "%d configs of the same workload, isValid + computeDistance, ref32 oracle, OpenMP" % sample,
            "one_core": {"value": 65536 / dt1, "unit": "configs/s", "cores": 1,
                         "sample": "the first 65,536 of those configs"}}
    return line, rv, rd


BAND_M = 1e-5   # FP32 rounding band of a decision margin (metres over error amplification)


def parity_accounting(eng, sid, robot, scene, q, outs, ref32):
    """Headline-size parity against the oracle (the checker, not the thing
    measured): the FP64 form against ref64, and every form against ref32, the
    reference's own FP32 numerics.  Each isValid flip and each distance
    difference above 1e-5 m against ref32 is listed with its FP64 decision
    margin (rpm_decision_margins), which must lie inside the FP32 rounding
    band."""
    import torch
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    rv32, rd32 = ref32
    rv64, rd64, _ = O.check_configs(robot, scene, q, prec="ref64", want=("valid", "dist"), nthreads=cores)
    out = {"configs": int(q.shape[0]), "band_m": BAND_M}
    v64, d64 = outs["fp64"]
    out["fp64_vs_ref64"] = {"isvalid_mismatches": int((v64 != rv64).sum()),
                            "distance_bit_mismatches": int((d64.view(np.uint64) != rd64.view(np.uint64)).sum())}
    v32, d32 = outs["fp32_recheck"]
    out["fp32_recheck_vs_ref64"] = {"isvalid_flips": int((v32 != rv64).sum()),
                                    "max_distance_error_m": float(np.abs(d32 - rd64).max())}
    vr, dr = outs["fp32_ref"]
    out["fp32_ref_vs_ref32"] = {"isvalid_mismatches": int((vr != rv32).sum()),
                                "distance_bit_mismatches": int((dr.view(np.uint64) != rd32.view(np.uint64)).sum())}
    for form in ("fp64", "fp32_recheck"):
        v, d = outs[form]
        flips = np.nonzero(v != rv32)[0]
        dflips = np.nonzero(np.abs(d - rd32) > 1e-5)[0]
        sel = np.union1d(flips, dflips)
        mv = md = np.zeros(0)
        if sel.size:
            qd = torch.from_numpy(np.ascontiguousarray(q[sel])).cuda()
            tv = torch.zeros(sel.size, dtype=torch.float64, device="cuda")
            tdm = torch.zeros(sel.size, dtype=torch.float64, device="cuda")
            eng.decision_margins(sid, qd, tv, tdm)
            eng.sync()
            mv, md = tv.cpu().numpy(), tdm.cpu().numpy()
        fm = mv[np.isin(sel, flips)]
        dm = md[np.isin(sel, dflips)]
        rest = np.setdiff1d(np.arange(q.shape[0]), dflips)
        out["%s_vs_ref32" % form] = {
            "isvalid_flips": int(flips.size), "max_flip_margin_m": float(fm.max()) if fm.size else None,
            "distance_diffs_gt_1e-5_m": int(dflips.size), "max_diff_margin_m": float(dm.max()) if dm.size else None,
            "all_inside_band": bool(np.all(fm < BAND_M) and np.all(dm < BAND_M)),
            "max_distance_diff_elsewhere_m": float(np.abs(d[rest] - rd32[rest]).max()) if rest.size else None,
            "flips": [{"config": int(c), "ours": int(v[c]), "ref32": int(rv32[c]), "margin_m": float(m)}
                      for c, m in zip(flips[:8], fm[:8])]}
    return out


def traffic_per_launch():
    path = os.path.join(ROOT, "profiles", "k_check_fp32_xarm6.json")
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_launch_full")
    except Exception:
        return None


def extra_workloads(eng, args):
    """The other configurations of the path, measured the same way (device
    events around whole steps, FP32 + FP64 recheck): edge checks (262,144
    spatial_10dof edges, 0.05 rad steps), the mixed-DOF profile launch
    (spatial 14/18/22, 500 AABBs) and the serving replay."""
    import torch
    from rpmplv2_gb300 import scenes, serve
    out = {}

    def timed(fn, steps=3, warmup=1):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    which = set(args.extra.split(","))
    if "planar" in which:
        out["planar_2dof"] = planar_line(eng, scenes, timed)
    if "edges" in which:
        out["edges"] = edges_line(eng, scenes, timed)
    if "mixed" in which:
        out["mixed_dof"] = mixed_line(eng, scenes, timed)
    if "large" in which:
        out["large_scene"] = large_line(eng, scenes, timed)
    if "serve" in which:
        out["serve"] = serve_line(eng, serve)
    if "planner" in which:
        out["planner"] = planner_line(eng, scenes, serve, timed)
    return out


def planner_line(eng, scenes, serve, timed):
    """The planner-side steps after the distance profile, each beside the oracle
    on one host core: the DRGBT horizon (computeReachedState of every horizon
    state, then computeDistance), MotionValidity::check with moving boxes, and
    RBT spines (extendSpine)."""
    import time
    import torch
    from oracle import oracle as O
    from rpmplv2_gb300 import _abi
    out = {}
    rng = np.random.default_rng(12)
    # ---- DRGBT horizon on the xarm6 workload
    robot, scene, q = scenes.xarm6_workload(4096, seed=13)
    sid = eng.create_scene(eng.upload_robot(robot), scene)
    _, d, _ = eng.check_configs_host(sid, q[:512], "fp32_recheck", want=("dist",))
    qc = torch.from_numpy(np.ascontiguousarray(q[int(np.argmax(d))])).cuda()
    for H in (10, 4096):
        hz = torch.from_numpy(scenes.uniform_configs(rng, H, 6)).cuda()
        qr = torch.zeros((H, 6), dtype=torch.float32, device="cuda")
        st = torch.zeros(H, dtype=torch.int32, device="cuda")
        dd = torch.zeros(H, dtype=torch.float64, device="cuda")
        ms = timed(lambda: eng.reached_states(sid, qc, hz, qr, st, dd, precision="fp32_ref"), steps=5, warmup=2)
        out["drgbt_horizon_%d" % H] = {"ms_per_call": ms, "states_per_s": H / (ms / 1e3)}
    hz10 = scenes.uniform_configs(rng, 10, 6)
    t0 = time.perf_counter()
    rq, _ = O.reached_states(robot, scene, qc.cpu().numpy(), hz10)
    O.check_configs(robot, scene, rq, prec="ref32", want=("dist",), nthreads=1)
    out["drgbt_horizon_10"]["cpu_ms"] = (time.perf_counter() - t0) * 1e3
    out["drgbt_horizon_10"]["workload"] = ("xarm6, 50 cubes + ground; 5 layers, NUM_ITER_SPINE 1, expanded bubble, "
                                           "D_CRIT 0.05, then computeDistance, all in the reference's numerics; "
                                           "cpu_ms: oracle, 1 core")
    eng.destroy_scene(sid)
    # ---- MotionValidity::check, spatial_10dof among 200 boxes, 5 of them moving at up to 1.6 m/s
    rb = serve.make_robot("spatial_10dof")
    sc = serve._scene_for(rb, rng, 200)
    idx = rng.choice(sc.n, 5, replace=False)
    mv = (_abi.MovingBox * 5)()
    for k, j in enumerate(idx):
        dim = rng.uniform(0.05, 0.2, 3).astype(np.float32)
        pos = rng.uniform(-0.8, 0.8, 3).astype(np.float32)
        sc.aabb[j] = scenes.box_aabb(dim, pos)
        sc.flags[j] |= _abi.RPM_OBS_DYNAMIC
        mv[k] = _abi.MovingBox(int(j), float(rng.uniform(0, 1.6)), tuple(dim), tuple(pos), (0.0, 0.0, 0.0, 1.0))
    sid = eng.create_scene(eng.upload_robot(rb), sc)
    M, N = 4096, 8   # NUM_VALIDITY_POINTS_CHECK = ceil(1.6 m/s x 0.05 s / 0.01 m)
    q1 = scenes.uniform_configs(rng, M, 10)
    q2 = (q1 + rng.uniform(-0.3, 0.3, q1.shape)).astype(np.float32)
    q1d, q2d = torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda()
    v = torch.zeros(M, dtype=torch.uint8, device="cuda")
    kk = torch.zeros(M, dtype=torch.int32, device="cuda")
    ms = timed(lambda: eng.motion_validity(sid, q1d, q2d, mv, 0.05, N, v, kk, precision="fp32_ref"), steps=5, warmup=2)
    t0 = time.perf_counter()
    O.motion_validity(rb, sc, q1[:256], q2[:256], mv, 0.05, N, prec="ref32")
    cpu_s = (time.perf_counter() - t0) / 256
    out["motion_validity"] = {"workload": "spatial_10dof among 200 boxes, 5 moving straight, 4,096 motions x 8 checks, "
                                          "reference numerics", "motions_per_s": M / (ms / 1e3), "ms_per_step": ms,
                              "valid_fraction": float(v.float().mean()), "cpu_motions_per_s": 1.0 / cpu_s}
    eng.destroy_scene(sid)
    # ---- RBT spines (xarm6, 5 iterations, expanded bubble)
    robot = serve.make_robot("xarm6")
    C = 65536
    qs = scenes.uniform_configs(rng, C, 6)
    qe = scenes.uniform_configs(rng, C, 6)
    prof = rng.uniform(0.01, 0.4, (C, 6)).astype(np.float32)
    dist = prof.min(axis=1).astype(np.float32)
    rid = eng.upload_robot(robot)
    tq, te, td, tp = (torch.from_numpy(a).cuda() for a in (qs, qe, dist, prof))
    qn = torch.zeros((C, 6), dtype=torch.float32, device="cuda")
    stt = torch.zeros(C, dtype=torch.int32, device="cuda")
    ms = timed(lambda: eng.extend_spines(rid, tq, te, td, tp, qn, stt, num_iter=5), steps=5, warmup=2)
    t0 = time.perf_counter()
    O.extend_spines(robot, qs[:4096], qe[:4096], dist[:4096], prof[:4096], num_iter=5)
    cpu_s = (time.perf_counter() - t0) / 4096
    out["spines"] = {"workload": "xarm6 extendSpine, 65,536 spines, NUM_ITER_SPINE 5, expanded bubble",
                     "spines_per_s": C / (ms / 1e3), "ms_per_step": ms, "cpu_spines_per_s": 1.0 / cpu_s}
    return out


def cpu_rates(run, total, n1, nall, unit, what):
    """CPU baseline columns: the oracle timed on the host, one core on the
    first n1 units and every core on the first nall units (bounded samples of
    the same workload)."""
    cores = os.cpu_count() or 1
    n1, nall = min(n1, total), min(nall, total)
    run(0, min(64, n1), 1)   # warm-up
    t0 = time.perf_counter()
    run(0, n1, 1)
    t1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    run(0, nall, cores)
    ta = time.perf_counter() - t0
    return {"one_core": n1 / t1, "all_cores": nall / ta, "cores": cores, "unit": unit,
            "sample": "%s; %d units on 1 core, %d on %d cores" % (what, n1, nall, cores)}


def planar_line(eng, scenes, timed):
    """planar_2dof, the plain FP64 form: 65,536 configurations against 4 AABBs, isValid + distance."""
    import torch
    from oracle import oracle as O
    robot, scene, q = scenes.planar_2dof_workload(65536, seed=0)
    sid = eng.create_scene(eng.upload_robot(robot), scene)
    qd = torch.from_numpy(q).cuda()
    C = q.shape[0]
    v = torch.zeros(C, dtype=torch.uint8, device="cuda")
    d = torch.zeros(C, dtype=torch.float64, device="cuda")
    ms = timed(lambda: eng.check_configs(sid, qd, "fp64", v, d, None), steps=5, warmup=3)
    rv, rd, _ = O.check_configs(robot, scene, q, prec="ref64", want=("valid", "dist"), nthreads=os.cpu_count() or 1)
    line = {"workload": "planar_2dof (r 0) vs 4 AABBs in a 2 m disk, 65,536 configs, isValid + computeDistance",
            "configs_per_s": C / (ms / 1e3), "ms_per_step": ms, "precision": "fp64",
            "isvalid_mismatches_vs_ref64": int((v.cpu().numpy() != rv).sum()),
            "distance_bit_mismatches_vs_ref64": int((d.cpu().numpy().view(np.uint64) != rd.view(np.uint64)).sum())}
    line["cpu"] = cpu_rates(lambda a, b, nt: O.check_configs(robot, scene, q[a:b], prec="ref64",
                                                             want=("valid", "dist"), nthreads=nt),
                            C, 65536, 65536, "configs/s", "isValid + distance, ref64 oracle")
    eng.destroy_scene(sid)
    return line


def edges_line(eng, scenes, timed):
    """262,144 spatial_10dof edges at 0.05 rad steps against 200 boxes."""
    import torch
    from oracle import oracle as O
    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(1 << 18, seed=2)
    sid = eng.create_scene(eng.upload_robot(robot), scene)
    q1d, q2d = torch.from_numpy(q1).cuda(), torch.from_numpy(q2).cuda()
    v = torch.zeros(q1.shape[0], dtype=torch.uint8, device="cuda")
    k = torch.zeros(q1.shape[0], dtype=torch.int32, device="cuda")
    shape = eng.autotune_edges(sid, q1d, q2d, v, step=float(step), precision="fp32_recheck", reps=2)
    eng.set_graphs(True)
    ms = timed(lambda: eng.check_edges(sid, q1d, q2d, v, k, step=float(step), precision="fp32_recheck"))
    eng.set_graphs(False)
    launched = eng.last_shape()
    checks = int(k.sum().item())
    line = {"workload": "spatial_10dof (r 0.03) vs 200 rotated boxes as fcl AABBs, 262,144 edges, 0.05 rad",
            "edges_per_s": q1.shape[0] / (ms / 1e3), "checks_per_s": checks / (ms / 1e3),
            "ms_per_step": ms, "checks_reference_order": checks, "valid_fraction": float(v.float().mean()),
            "tile_shape": shape, "launched_shape": launched, "cuda_graph": True, "precision": "fp32_recheck"}
    line["cpu"] = cpu_rates(lambda a, b, nt: O.check_edges(robot, scene, q1[a:b], q2[a:b], step=float(step), prec="ref32",
                                                           nthreads=nt),
                            q1.shape[0], 2048, 32768, "edges/s", "edge checks in reference order, ref32 oracle")
    eng.destroy_scene(sid)
    return line


def mixed_line(eng, scenes, timed):
    """Per-link distance profiles of spatial 14/18/22-DOF chains against 500 AABBs in one launch."""
    import torch
    from oracle import oracle as O
    scene, parts = scenes.mixed_dof_workload(seed=3)
    items = []
    for robot, q in parts:
        sid = eng.create_scene(eng.upload_robot(robot), scene)
        C, L = q.shape[0], robot.num_links
        items.append((sid, torch.from_numpy(q).cuda(), None, torch.zeros(C, dtype=torch.float64, device="cuda"),
                      torch.zeros((C, L), device="cuda")))
    total = sum(it[1].shape[0] for it in items)
    ms = timed(lambda: eng.check_batch(items, "fp32_recheck"))
    line = {"workload": "spatial 14/18/22 DOF (r 0.03), 32,768/49,152/49,152 configs, 500 AABBs, "
                        "per-link distance + global min in one launch",
            "configs_per_s": total / (ms / 1e3), "ms_per_step": ms, "precision": "fp32_recheck"}
    # the CPU columns on the 18-DOF part, the middle of the three
    robot18, q18 = parts[1]
    line["cpu"] = cpu_rates(lambda a, b, nt: O.check_configs(robot18, scene, q18[a:b], prec="ref32",
                                                             want=("dist", "profile"), nthreads=nt),
                            q18.shape[0], 256, 4096, "configs/s", "spatial_18dof part, distance + profile, ref32 oracle")
    for it in items:
        eng.destroy_scene(it[0])
    return line


def large_line(eng, scenes, timed):
    """isValid + computeDistance of 65,536 spatial_22dof configurations against 1000 boxes (the
    warp-per-configuration layout), the size of the largest serving requests."""
    import torch
    robot, scene, q = scenes.large_scene_workload(65536, seed=6)
    sid = eng.create_scene(eng.upload_robot(robot), scene)
    qd = torch.from_numpy(q).cuda()
    C = q.shape[0]
    v = torch.zeros(C, dtype=torch.uint8, device="cuda")
    d = torch.zeros(C, dtype=torch.float64, device="cuda")
    shape = eng.autotune_configs(sid, qd, "fp32_recheck", v, d, reps=2)
    ms = timed(lambda: eng.check_configs(sid, qd, "fp32_recheck", v, d, None), steps=5, warmup=2)
    line = {"workload": "spatial_22dof (r 0.03) vs 1000 boxes (dims U[0.02, 0.15] m, 1.5 m ball), 65,536 configs, "
                        "isValid + computeDistance",
            "configs_per_s": C / (ms / 1e3), "ms_per_step": ms, "valid_fraction": float(v.float().mean()),
            "tile_shape": shape, "launched_shape": eng.last_shape(), "precision": "fp32_recheck"}
    eng.destroy_scene(sid)
    return line


def serve_line(eng, serve):
    """The serving replay: 20,000 requests/s for 0.5 s over 64 resident scenes."""
    wl = serve.serving_workload(eng, seed=4, rate=20000.0, duration=0.5)
    srv = serve.Server(eng)   # the library's defaults (rpm_server_config)
    srv.replay(wl["requests"][:200], [0.0] * 200)
    tim = srv.replay(wl["requests"], wl["arrivals"], wl["motions"], period=0.001)
    summ = serve.latency_summary(tim, wl["meta"])
    summ.update({"workload": "64 resident scenes (robots of configs 0-3, 10-1000 boxes log-uniform, 20% with 5 "
                             "boxes moving up to 1.6 m/s updated every 1 ms), Poisson 20,000 req/s for 0.5 s, "
                             "sizes log-uniform 1-65,536, isValid / distance / edge in equal shares, of which 10% "
                             "replaced by DRGBT steps (horizon of reached states, MotionValidity with moving boxes)",
                 "memory_budget_bytes": 8 << 30, "bulk_slots": 4, "express_slots": 24, "express_work": 8192,
                 "chunk_work": 65536, "bulk_sms": "all but 48 (green context)"})
    # capacity: the same trace submitted at once; latency at a rate the engine sustains
    t = srv.replay(wl["requests"], [0.0] * len(wl["requests"]))
    summ["capacity_req_per_s"] = len(t) / max(x.t_done for x in t)
    srv.close()
    for sid in wl["scene_ids"]:
        eng.destroy_scene(sid)
    # the 12,000 req/s trace on a server of its own (not one just drained of a saturating burst)
    wl12 = serve.serving_workload(eng, seed=5, rate=12000.0, duration=0.5)
    srv = serve.Server(eng)
    srv.replay(wl12["requests"][:200], [0.0] * 200)
    t12 = srv.replay(wl12["requests"], wl12["arrivals"], wl12["motions"], period=0.001)
    s12 = serve.latency_summary(t12, wl12["meta"])
    summ["at_12000_req_per_s"] = {k: s12[k] for k in ("queries_per_s", "p50_ms", "p99_ms", "p50_ms_4096", "p99_ms_4096",
                                                      "p99_ms_4096_configs", "bucket_4096_by_kind", "p99_ms_le4096",
                                                      "median_run_ms", "drgbt_horizon", "motion_validity")}
    wl = wl12
    srv.close()
    for sid in wl["scene_ids"]:
        eng.destroy_scene(sid)
    return summ


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from rpmplv2_gb300 import scenes
    robot, scene, q = scenes.xarm6_workload(args.configs, seed=1)
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    sample = min(args.configs, 1 << 18)
    for w in range(args.warmup):
        O.check_configs(robot, scene, q[:4096], prec="ref32", nthreads=cores)
    times = []
    for k in range(args.steps):
        qs = np.ascontiguousarray(q[(k * sample) % args.configs:][:sample])
        t0 = time.perf_counter()
        O.check_configs(robot, scene, qs, prec="ref32", nthreads=cores)
        times.append(time.perf_counter() - t0)
    value = sample * len(times) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "configs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_per_step": sample,
                       "implementation": "CPU restatement of the reference's RealVectorSpace path (ref32)"},
            "cpu_baseline": {"value": value, "unit": "configs/s", "cores": cores, "kind": "port",
                             "sample": "%d configs per step, isValid + computeDistance" % sample},
            "e2e": {"value": value, "unit": "configs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    from rpmplv2_gb300 import scenes
    from rpmplv2_gb300.engine import Engine

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    C = args.configs
    robot, scene, q = scenes.xarm6_workload(C, seed=1 + rank)
    eng = Engine(local)
    rid = eng.upload_robot(robot)
    sid = eng.create_scene(rid, scene)
    qd = torch.from_numpy(q).cuda()
    valid = torch.zeros(C, dtype=torch.uint8, device="cuda")
    distv = torch.zeros(C, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            eng.check_configs(sid, qd, prec, valid, distv)
        eng.set_timing(True)
        barrier()
        step_ms, bulk_ms, re_ms, rechecked = [], [], [], []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            eng.check_configs(sid, qd, prec, valid, distv)
            b.record()
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
            bm, rm = eng.last_timing()
            bulk_ms.append(bm)
            re_ms.append(rm)
            rechecked.append(eng.stats()["rechecked"])
        barrier()
        eng.set_timing(False)
        return step_ms, bulk_ms, re_ms, rechecked

    # ---- headline: FP32 + FP64 recheck, inputs resident in HBM
    peak_fp32 = eng.fp32_peak_tflops()
    with ClockSampler(local) as clk:
        step_ms, bulk_ms, re_ms, rechecked = timed("fp32_recheck", args.steps, args.warmup)
    clocks = clk.summary()
    v32, d32 = valid.clone(), distv.clone()
    # ---- the plain FP64 form on the same batch
    step64, bulk64, _, _ = timed("fp64", max(2, min(args.steps, 3)), 1)
    v64, d64 = valid.clone(), distv.clone()
    flips = int((v32 != v64).sum().item())
    max_derr = float((d32 - d64).abs().max().item())
    # ---- the reference-numerics form on the same batch (bit-equal to ref32)
    stepref, _, _, _ = timed("fp32_ref", 2, 1)
    outs = {"fp32_recheck": (v32.cpu().numpy(), d32.cpu().numpy()), "fp64": (v64.cpu().numpy(), d64.cpu().numpy()),
            "fp32_ref": (valid.cpu().numpy(), distv.cpu().numpy())}

    t_local = sum(step_ms) / 1e3
    if dist is not None:
        t = torch.tensor([t_local], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_local = float(t.item())
    value = ws * C * args.steps / t_local
    fp64_value = C / (statistics.median(step64) / 1e3)

    # ---- end to end through the host-buffer C ABI call, pinned host memory
    qh = torch.from_numpy(q).pin_memory().numpy()
    vh = torch.zeros(C, dtype=torch.uint8).pin_memory().numpy()
    dh = torch.zeros(C, dtype=torch.float64).pin_memory().numpy()
    import ctypes
    lib = eng.lib
    for _ in range(2):
        lib.rpm_check_configs_host(eng.ctx, sid, 1, qh.ctypes.data, C, vh.ctypes.data, dh.ctypes.data, None)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc = lib.rpm_check_configs_host(eng.ctx, sid, 1, qh.ctypes.data, C, vh.ctypes.data, dh.ctypes.data, None)
        if rc != 0:
            raise RuntimeError("rpm_check_configs_host failed: %s" % lib.rpm_last_error_string().decode())
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_ok = bool(np.array_equal(vh, v32.cpu().numpy()))

    # ---- roofline of the dominant kernel (the FP32 bulk pass)
    bulk_s = statistics.median(bulk_ms) / 1e3
    achieved = FLOP_PER_CONFIG * C / bulk_s / 1e12
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    hbm_achieved = BYTES_PER_CONFIG * C / bulk_s / 1e9

    extra = {} if args.no_extra else extra_workloads(eng, args)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "configs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 recheck)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "global_batch": C * ws, "precision": "fp32_recheck",
                   "l2": "flushed (256 MB write) between timed steps", "parallelism": "replicas, configs sharded"},
        "fp64": {"value": fp64_value, "unit": "configs/s", "ms_per_step": statistics.median(step64),
                 "speedup_fp32_recheck_over_fp64": value / ws / fp64_value, "isvalid_flips": flips,
                 "max_distance_diff_m": max_derr},
        "recheck": {"configs_per_step": int(statistics.median(rechecked)),
                    "fraction": statistics.median(rechecked) / C, "kernel_ms": statistics.median(re_ms),
                    "note": "FP64 rechecks of a step, once per output pass (isValid, distance) that needed one; "
                            "kernel_ms: the recheck round after the last main launch"},
        "clocks": clocks,
        "e2e": {"value": C * args.steps / e2e_s, "unit": "configs/s", "h2d_bytes_per_step": C * D * 4,
                "d2h_bytes_per_step": C * (1 + 8), "call": "rpm_check_configs_host", "matches_device_run": e2e_ok,
                "transfer": "pinned host buffers, staged through device memory by DMA copies in one chunk of "
                            "up to 1,048,576 configurations"},
        # per step: the check order (k_bin_count, k_bin_scan, k_bin_scatter), k_check_fp32 compiled
        # for each of the two outputs (isValid, distance), then one recheck round for both:
        # k_pair_skel / k_pair_key / k_pair_scatter / k_pair_eval / k_pair_fold and the
        # whole-configuration k_recheck
        "gpu_launches": 11 * args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                     "frac": achieved / peak_fp32 if peak_fp32 else None, "traffic": traffic_per_launch(),
                     "kernel": "k_check_fp32", "kernel_ms": statistics.median(bulk_ms),
                     "flop_per_config": FLOP_PER_CONFIG,
                     "peak_source": "FFMA probe measured in this run (rpm_probe_fp32_peak)",
                     "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": (hbm_achieved / hbm_peak) if hbm_peak else None,
                             "bytes_per_config": BYTES_PER_CONFIG, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}},
    }
    line.update(extra)
    line["fp32_ref_form"] = {"value": C / (statistics.median(stepref) / 1e3), "unit": "configs/s",
                             "note": "the reference's own numerics on the device (FP64 FK rounded to FP32, FP32 trees)"}
    if ws == 1 or rank == 0:
        line["cpu_baseline"], rv32, rd32 = cpu_baseline(robot, scene, q, min(C, 1 << 20))
        n = rv32.shape[0]
        line["parity"] = parity_accounting(eng, sid, robot, scene, q[:n], {k: (a[:n], b[:n]) for k, (a, b) in outs.items()},
                                           (rv32, rd32))
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
