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


ADV_COLL, ADV_DIST, ADV_SEGSEG = 0, 1, 2


def adversarial_cases(seed, per_kind=1500):
    """Directed cases for the branches uniform sampling almost never reaches:
    degenerate (zero-length) segments, axis-parallel segments lying in face
    planes or collinear with box edges, endpoints exactly on face planes,
    edges and corners, segments at exactly r and r*sqrt(3)/3 from a face,
    face crossings on a rectangle's border, clearances at the
    EQUALITY_THRESHOLD snap, and for distanceLineSegToLineSeg
    (CollisionAndDistance.cpp:217-320) parallel, collinear, degenerate,
    crossing and near-threshold segment pairs (the NaN-s path of :223-230).

    Returns (A, B, X, r, kind): X is the AABB for kinds 0 (collision) and 1
    (distance), and the second segment (C, D) for kind 2."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    rows = []

    def box():
        c = rng.uniform(-0.3, 0.3, 3).astype(f32)
        h = rng.uniform(0.01, 0.2, 3).astype(f32)
        return np.concatenate([c - h, c + h]).astype(f32)

    def near(o, spread=0.3):
        lo, hi = o[:3] - spread, o[3:] + spread
        return rng.uniform(lo, hi).astype(f32)

    radii = (0.0, 0.02, 0.05, 0.12)
    for it in range(per_kind):
        o = box()
        r = f32(radii[it % 4])
        rn = f32(np.float64(r) * np.sqrt(3.0) / 3)   # the reference's r_new rounding
        g = it % 12
        ax = int(rng.integers(3))
        side = int(rng.integers(2))
        face = o[ax + 3 * side]
        a, b = near(o), near(o)
        if g == 0:                                    # zero-length segment
            b = a.copy()
        elif g == 1:                                  # zero-length on a face plane
            a[ax] = face
            b = a.copy()
        elif g == 2:                                  # axis-parallel, fixed coordinates on face planes or offsets
            offs = (f32(0), r, -r, rn, -rn)
            for k in range(3):
                if k != ax:
                    a[k] = f32(o[k + 3 * int(rng.integers(2))] + offs[int(rng.integers(len(offs)))])
                    b[k] = a[k]
        elif g == 3:                                  # lying in a face plane
            a[ax] = b[ax] = face
        elif g == 4:                                  # collinear with a box edge
            for k in range(3):
                if k != ax:
                    a[k] = b[k] = o[k + 3 * int(rng.integers(2))]
        elif g == 5:                                  # endpoint on a corner
            a = np.array([o[k + 3 * int(rng.integers(2))] for k in range(3)], f32)
        elif g == 6:                                  # endpoint on an edge
            for k in range(3):
                if k != ax:
                    a[k] = o[k + 3 * int(rng.integers(2))]
        elif g == 7:                                  # parallel to a face at exactly r or r_new
            d = (r, rn)[int(rng.integers(2))]
            a[ax] = b[ax] = f32(face + d) if side else f32(face - d)
        elif g == 8:                                  # crossing a face on its rectangle's border
            m = near(o, 0.0)
            m[ax] = face
            k2 = (ax + 1 + int(rng.integers(2))) % 3
            m[k2] = o[k2 + 3 * int(rng.integers(2))]
            dv = rng.normal(0, 0.1, 3).astype(f32)
            dv[ax] = f32(abs(dv[ax]) + 0.01)
            a, b = (m + dv).astype(f32), (m - dv).astype(f32)
        elif g == 9:                                  # clearance at the EQUALITY_THRESHOLD snap
            eps = f32(1e-4) + f32(rng.choice([-2e-7, -6e-8, 0.0, 6e-8, 2e-7]))
            off = f32(r + eps)
            a[ax] = b[ax] = f32(face + off) if side else f32(face - off)
        elif g == 10:                                 # an endpoint inside the box
            a = rng.uniform(o[:3], o[3:]).astype(f32)
        else:                                         # beyond a corner region, parallel to an edge
            for k in range(3):
                s = int(rng.integers(2))
                a[k] = f32(o[k + 3 * s] + (0.05 if s else -0.05) * rng.uniform(0.1, 1.0))
            b = a.copy()
            b[ax] = f32(a[ax] + rng.uniform(-0.4, 0.4))
        kind = ADV_COLL if it % 2 == 0 else ADV_DIST
        rows.append((a, b, o, r, kind))
        rows.append((a, b, o, r, 1 - kind))
    for it in range(per_kind):
        g = it % 8
        a = rng.uniform(-0.5, 0.5, 3).astype(f32)
        u = rng.normal(0, 0.2, 3).astype(f32)
        if it % 3 == 0:                               # axis-aligned directions, as box edges are
            u = np.zeros(3, f32)
            u[int(rng.integers(3))] = f32(rng.uniform(0.05, 0.4))
        b = (a + u).astype(f32)
        if g == 0:                                    # parallel, offset
            off = rng.normal(0, 0.05, 3).astype(f32)
            lam = f32(rng.choice([1.0, -1.0, 2.0, 0.5]))
            c = (a + off).astype(f32)
            d = (c + lam * u).astype(f32)
        elif g == 1:                                  # collinear, overlapping or disjoint
            t1, t2 = (f32(x) for x in rng.choice([-0.5, 0.0, 0.25, 0.5, 1.0, 1.5, 2.0], 2, replace=False))
            c, d = (a + t1 * u).astype(f32), (a + t2 * u).astype(f32)
        elif g == 2:                                  # first segment degenerate
            b = a.copy()
            c = rng.uniform(-0.5, 0.5, 3).astype(f32)
            d = (c + rng.normal(0, 0.2, 3)).astype(f32)
        elif g == 3:                                  # second segment degenerate
            c = rng.uniform(-0.5, 0.5, 3).astype(f32)
            d = c.copy()
        elif g == 4:                                  # both degenerate (same or distinct points)
            b = a.copy()
            c = a.copy() if it % 16 == 4 else rng.uniform(-0.5, 0.5, 3).astype(f32)
            d = c.copy()
        elif g == 5:                                  # crossing at an interior point
            m = (a + f32(0.5) * u).astype(f32)
            w = rng.normal(0, 0.2, 3).astype(f32)
            c, d = (m - w).astype(f32), (m + w).astype(f32)
        elif g == 6:                                  # perpendicular at the snap distance
            n = np.cross(u, rng.normal(0, 1, 3)).astype(f32)
            n = (n / np.linalg.norm(n)).astype(f32)
            w = np.cross(u, n).astype(f32)
            dd = f32(1e-4) + f32(rng.choice([-2e-7, 0.0, 2e-7, 1e-6]))
            m = (a + f32(0.5) * u + dd * n).astype(f32)
            c, d = (m - f32(0.5) * w).astype(f32), (m + f32(0.5) * w).astype(f32)
        else:                                         # shared endpoint
            c = b.copy()
            d = (c + rng.normal(0, 0.2, 3)).astype(f32)
        rows.append((a, b, np.concatenate([c, d]).astype(f32), f32(0), ADV_SEGSEG))
    A = np.array([x[0] for x in rows], f32)
    B = np.array([x[1] for x in rows], f32)
    X = np.array([x[2] for x in rows], f32)
    r = np.array([x[3] for x in rows], f32)
    kind = np.array([x[4] for x in rows], np.int32)
    return A, B, X, r, kind


def adversarial_fixture(seed):
    """The directed cases with their answers: adv_reference from the
    reference's own CollisionAndDistance.cpp (when its tree is present),
    adv_ref32 / adv_ref64 from the oracle.  adv_undefined marks distance cases
    that reach the reference's uninitialised edge matrix in getLineSegments
    (:542-574 selecting no edge): the reference's answer there is whatever the
    heap held, so those cases pin only the library's documented choice
    ("no edge", the oracle's answer)."""
    import ctypes
    A, B, X, r, kind = adversarial_cases(seed)
    n = len(r)
    ref32 = np.zeros(n, np.float64)
    ref64 = np.zeros(n, np.float64)
    undefined = np.zeros(n, np.uint8)
    fp = ctypes.POINTER(ctypes.c_float)
    P = lambda a: np.ascontiguousarray(a).ctypes.data_as(fp)
    L = O.lib()
    O.undefined_hits()
    for i in range(n):
        if kind[i] == ADV_COLL:
            ref32[i] = O.prim_collision(A[i], B[i], r[i], X[i], "ref32")
            ref64[i] = O.prim_collision(A[i], B[i], r[i], X[i], "ref64")
        elif kind[i] == ADV_DIST:
            ref32[i] = O.prim_distance(A[i], B[i], r[i], X[i], "ref32")[0]
            ref64[i] = O.prim_distance(A[i], B[i], r[i], X[i], "ref64")[0]
            undefined[i] = 1 if O.undefined_hits() else 0
        else:
            ref32[i] = L.orc_prim_segseg(P(A[i]), P(B[i]), P(X[i][:3]), P(X[i][3:]), 32, None)
            ref64[i] = L.orc_prim_segseg(P(A[i]), P(B[i]), P(X[i][:3]), P(X[i][3:]), 64, None)
    out = {"adv_A": A, "adv_B": B, "adv_X": X, "adv_r": r, "adv_kind": kind, "adv_undefined": undefined,
           "adv_ref32": ref32, "adv_ref64": ref64}
    R = O.ref()
    if R is not None:
        refv = np.zeros(n, np.float64)
        for i in range(n):
            if kind[i] == ADV_COLL:
                refv[i] = R.ref_collision(P(A[i]), P(B[i]), float(r[i]), P(X[i]))
            elif kind[i] == ADV_DIST:
                refv[i] = R.ref_distance(P(A[i]), P(B[i]), float(r[i]), P(X[i]), None, None)
            else:
                refv[i] = R.ref_segseg(P(A[i]), P(B[i]), P(X[i][:3]), P(X[i][3:]))
        out["adv_reference"] = refv
    return out


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
    out.update(adversarial_fixture(seed=105))
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
