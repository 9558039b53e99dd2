"""Generates tests/golden/golden.npz: small seeded inputs of every workload shape
with the oracle's outputs in both numerics, plus primitive cases answered by
the reference's own CollisionAndDistance.cpp (compiled in place from the
reference tree by oracle/build.py) when that tree is present.

python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from rpmplv2_gb300 import scenes  # noqa: E402


def primitive_cases(n, seed):
    """Segments near random boxes, including axis-parallel segments and
    endpoints on face planes (the branch-heavy corners of the trees)."""
    rng = np.random.default_rng(seed)
    A = np.zeros((n, 3), np.float32)
    B = np.zeros((n, 3), np.float32)
    obs = np.zeros((n, 6), np.float32)
    r = np.zeros(n, np.float32)
    for it in range(n):
        c = rng.uniform(-0.3, 0.3, 3).astype(np.float32)
        h = rng.uniform(0.01, 0.2, 3).astype(np.float32)
        o = np.concatenate([c - h, c + h]).astype(np.float32)
        a = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        b = (a + rng.normal(0, 0.1, 3)).astype(np.float32) if it % 3 == 0 else rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        if it % 7 == 0:
            b[it % 3] = a[it % 3]
        if it % 11 == 0:
            a[(it // 11) % 3] = o[(it // 11) % 3]
        A[it], B[it], obs[it] = a, b, o
        r[it] = rng.choice([0.0, 0.02, 0.05, 0.12])
    return A, B, obs, r


def main():
    out = {}
    robot, scene, q = scenes.planar_2dof_workload(4096, seed=100)
    out["planar_q"], out["planar_aabb"] = q, scene.aabb
    for prec in ("ref32", "ref64"):
        v, d, p = O.check_configs(robot, scene, q, prec=prec)
        out["planar_%s_valid" % prec], out["planar_%s_dist" % prec], out["planar_%s_prof" % prec] = v, d, p

    robot, scene, q = scenes.xarm6_workload(2048, seed=101)
    out["xarm6_q"], out["xarm6_aabb"], out["xarm6_tol"], out["xarm6_flags"] = q, scene.aabb, scene.tol, scene.flags
    for prec in ("ref32", "ref64"):
        v, d, p = O.check_configs(robot, scene, q, prec=prec)
        out["xarm6_%s_valid" % prec], out["xarm6_%s_dist" % prec], out["xarm6_%s_prof" % prec] = v, d, p
    out["xarm6_skel64"] = O.skeleton(robot, q[:64], prec="ref64")
    out["xarm6_skel32"] = O.skeleton(robot, q[:64], prec="ref32")

    robot, scene, q1, q2, step = scenes.spatial10_edge_workload(512, seed=102)
    out["edges_q1"], out["edges_q2"], out["edges_aabb"] = q1, q2, scene.aabb
    for prec in ("ref32", "ref64"):
        v, k = O.check_edges(robot, scene, q1, q2, step=step, prec=prec)
        out["edges_%s_valid" % prec], out["edges_%s_checks" % prec] = v, k

    scene, parts = scenes.mixed_dof_workload(counts=(256, 256, 256), seed=103)
    out["mixed_aabb"] = scene.aabb
    for robot, q in parts:
        tag = "mixed%d" % robot.num_dofs
        out[tag + "_q"] = q
        v, d, p = O.check_configs(robot, scene, q, prec="ref64")
        out[tag + "_ref64_valid"], out[tag + "_ref64_dist"], out[tag + "_ref64_prof"] = v, d, p

    A, B, obs, r = primitive_cases(4000, seed=104)
    out["prim_A"], out["prim_B"], out["prim_obs"], out["prim_r"] = A, B, obs, r
    coll = np.array([O.prim_collision(A[i], B[i], r[i], obs[i], "ref32") for i in range(len(r))], np.uint8)
    dist = np.array([O.prim_distance(A[i], B[i], r[i], obs[i], "ref32")[0] for i in range(len(r))], np.float32)
    out["prim_ref32_coll"], out["prim_ref32_dist"] = coll, dist
    R = O.ref()
    if R is not None:
        import ctypes
        fp = ctypes.POINTER(ctypes.c_float)
        P = lambda a: np.ascontiguousarray(a).ctypes.data_as(fp)
        rc = np.array([R.ref_collision(P(A[i]), P(B[i]), float(r[i]), P(obs[i])) for i in range(len(r))], np.uint8)
        rd = np.array([R.ref_distance(P(A[i]), P(B[i]), float(r[i]), P(obs[i]), None, None) for i in range(len(r))],
                      np.float32)
        out["prim_reference_coll"], out["prim_reference_dist"] = rc, rd
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
