"""The warp sincos (rpm_dev.cuh: warp_sincos) evaluates the sine and cosine
polynomials of taylor_sincos as one instruction stream: the sine's Horner
recurrence starts one step earlier from 0 (z * 0 + c0 is c0), the
coefficients and the last factor are selected per lane, and the quadrant swap
trades the two values.  This restates both sequences in IEEE double (numpy
float64 scalars: every product and sum rounded, no fused multiply-add, as
dmul/dadd are on the device) and checks that they give the same bits.  So
does the warp forward kinematics' joint step (skel_coop), branchy against
branch-free with selected operands.  The GPU tests check the device code
itself through the skeletons built on it."""
import numpy as np

F = np.float64
TWO_OVER_PI = F.fromhex("0x1.45f306dc9c883p-1")
P1, P2, P3 = F.fromhex("0x1.921fb54400000p+0"), F.fromhex("0x1.0b4611a600000p-34"), F.fromhex("0x1.3198a2e037073p-69")
SIN = [F.fromhex(h) for h in ("0x1.952c77030ad4ap-49", "-0x1.ae7f3e733b81fp-41", "0x1.6124613a86d09p-33",
                              "-0x1.ae64567f544e4p-26", "0x1.71de3a556c734p-19", "-0x1.a01a01a01a01ap-13",
                              "0x1.1111111111111p-7", "-0x1.5555555555555p-3")]
COS = [F.fromhex(h) for h in ("-0x1.6827863b97d97p-53", "0x1.ae7f3e733b81fp-45", "-0x1.93974a8c07c9dp-37",
                              "0x1.1eed8eff8d898p-29", "-0x1.27e4fb7789f5cp-22", "0x1.a01a01a01a01ap-16",
                              "-0x1.6c16c16c16c17p-10", "0x1.5555555555555p-5", "-0x1.0000000000000p-1")]


def _reduce(x):
    kd = np.rint(x * TWO_OVER_PI)
    r = x + -(kd * P1)
    r = r + -(kd * P2)
    r = r + -(kd * P3)
    return kd, r, r * r


def per_lane(x):
    """taylor_sincos: both polynomials in one lane."""
    kd, r, z = _reduce(x)
    ps = SIN[0]
    for c in SIN[1:]:
        ps = c + z * ps
    s = r + (r * z) * ps
    pc = COS[0]
    for c in COS[1:]:
        pc = c + z * pc
    c = F(1.0) + z * pc
    q = int(kd) & 3
    return [(s, c), (c, -s), (-s, -c), (-c, s)][q]


def split(x):
    """warp_sincos: the sine lane and the cosine lane of one joint."""
    kd, r, z = _reduce(x)
    rz = r * z
    out = {}
    for is_sin in (True, False):
        p = F(0.0) if is_sin else COS[0]
        for k in range(8):
            p = (SIN[k] if is_sin else COS[k + 1]) + z * p
        out[is_sin] = (r if is_sin else F(1.0)) + (rz if is_sin else z) * p
    q = int(kd) & 3
    res = []
    for is_sin in (True, False):
        v, o = out[is_sin], out[not is_sin]
        base = o if q & 1 else v
        neg = (q & 2) != 0 if is_sin else q in (1, 2)
        res.append(-base if neg else base)
    return tuple(res)


def test_split_sincos_equals_per_lane_bits():
    rng = np.random.default_rng(7)
    xs = np.concatenate([rng.uniform(-np.pi, np.pi, 20000), rng.uniform(-50.0, 50.0, 5000),
                         np.float32(rng.uniform(-np.pi, np.pi, 5000)).astype(np.float64),
                         np.array([0.0, -0.0, np.pi / 4, -np.pi / 2, np.pi, 1e-30, -1e-8])])
    for x in xs:
        a, b = per_lane(F(x)), split(F(x))
        assert np.float64(a[0]).tobytes() == np.float64(b[0]).tobytes(), x
        assert np.float64(a[1]).tobytes() == np.float64(b[1]).tobytes(), x


def _joint(v, X_p, M, rot_identity, ax, sn, cs, branch_free):
    """One skel_coop joint for the 12 lanes (R row-major on lanes 0-8, p on
    9-11): the branchy per-lane form and the form with selected operands."""
    ia, ib = {0: (1, 2), 1: (2, 0), 2: (0, 1)}[ax]
    new = list(v)
    for lane in range(12):
        is_r, is_p = lane < 9, lane >= 9
        row, col = (lane // 3, lane % 3) if is_r else (lane - 9, 0)
        r0, r1, r2 = v[3 * row], v[3 * row + 1], v[3 * row + 2]
        if branch_free:
            X = (X_p[0], X_p[1], X_p[2]) if is_p else (M[col], M[3 + col], M[6 + col])
            t = (r0 * X[0] + r1 * X[1]) + r2 * X[2]
            tp = t + v[lane]
            new[lane] = tp if is_p else (t if (is_r and not rot_identity) else v[lane])
        elif is_p:
            new[lane] = ((r0 * X_p[0] + r1 * X_p[1]) + r2 * X_p[2]) + v[lane]
        elif not rot_identity:
            new[lane] = (r0 * M[col] + r1 * M[3 + col]) + r2 * M[6 + col]
    out = list(new)
    for lane in range(9):
        row, col = lane // 3, lane % 3
        x = new[3 * row + (ib if col == ia else ia)]
        if branch_free:
            a, b = col == ia, col == ib
            w = new[lane] * cs + x * (-sn if b else sn)
            out[lane] = w if (a or b) else new[lane]
        elif col == ia:
            out[lane] = new[lane] * cs + x * sn
        elif col == ib:
            out[lane] = new[lane] * cs + -(x * sn)
    return out


def test_branch_free_joint_equals_branchy_bits():
    rng = np.random.default_rng(11)
    for _ in range(3000):
        vals = rng.normal(size=24)
        vals[rng.random(24) < 0.2] = 0.0
        vals[rng.random(24) < 0.05] = -0.0
        v = [F(x) for x in vals[:12]]
        M = [F(x) for x in vals[12:21]]
        Xp = [F(x) for x in vals[21:24]]
        q = F(rng.uniform(-np.pi, np.pi)) if rng.random() < 0.9 else F(0.0)
        sn, cs = per_lane(q)
        ax, ident = int(rng.integers(0, 3)), bool(rng.random() < 0.3)
        a = _joint(v, Xp, M, ident, ax, sn, cs, False)
        b = _joint(v, Xp, M, ident, ax, sn, cs, True)
        assert all(np.float64(p).tobytes() == np.float64(r).tobytes() for p, r in zip(a, b))
