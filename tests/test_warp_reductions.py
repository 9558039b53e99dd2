"""Warp reductions that stand in for serial loops of the reference (rpm_spine.cuh:
extend_spine_warp's step, enclosing_rows_warp; rpm_exact.cu: k_reached_states's
underestimation), restated in float32 on the CPU: each gives the serial loop's
bits, including ties between +0 and -0 and NaN quotients."""
import numpy as np


def min_std(a, b):          # std::min: (b < a) ? b : a
    return b if b < a else a


def max_std(a, b):          # std::max: (a < b) ? b : a
    return b if a < b else a


def serial_step(x):
    step = np.float32(np.inf)
    for v in x:
        step = min_std(step, v)
    return step


def tree_step(x):
    """A value per lane (NaN as +inf), then five xor-shuffle rounds that take
    the smaller value and, on a tie, the lower lane."""
    val = [np.float32(np.inf)] * 32
    at = list(range(32))
    for i, v in enumerate(x):
        val[i] = np.float32(np.inf) if v != v else v
    off = 16
    while off:
        nv, na = val[:], at[:]
        for lane in range(32):
            y, ay = val[lane ^ off], at[lane ^ off]
            if y < val[lane] or (y == val[lane] and ay < at[lane]):
                nv[lane], na[lane] = y, ay
        val, at = nv, na
        off >>= 1
    return val[0]


def test_step_min_tree_keeps_the_serial_bits():
    rng = np.random.default_rng(3)
    pool = np.array([0.0, -0.0, np.nan, np.inf, 0.5, 0.25, -1.0, 2.0], np.float32)
    for _ in range(3000):
        D = int(rng.integers(1, 23))
        x = np.where(rng.random(D) < 0.5, rng.choice(pool, D), rng.normal(size=D).astype(np.float32)).astype(np.float32)
        a, b = serial_step(x), tree_step(x)
        assert np.float32(a).tobytes() == np.float32(b).tobytes(), x


def test_enclosing_rows_prefix_max_equals_serial_rows():
    """enclosing_row's running max over the columns, against its terms laid
    out per (joint, column) with zeros where the row adds none, then one
    running max per row: max is exact on these non-negative terms."""
    rng = np.random.default_rng(4)
    for _ in range(500):
        D = int(rng.integers(2, 23))
        terms = np.abs(rng.normal(size=(D, D + 1))).astype(np.float32)
        terms[rng.random((D, D + 1)) < 0.3] = 0.0
        for i in range(D):
            terms[i, :i + 1] = 0.0
        serial = np.zeros((D, D + 1), np.float32)
        for i in range(D):
            for j in range(i + 1, D + 1):
                if terms[i, j] != 0.0:
                    serial[i, j] = max_std(serial[i, j - 1], terms[i, j])
                else:
                    serial[i, j] = serial[i, j - 1]
        warp = np.zeros_like(serial)
        for i in range(D):
            r = np.float32(0.0)
            for j in range(D + 1):
                r = max_std(r, terms[i, j])
                warp[i, j] = r
        assert serial.tobytes() == warp.tobytes()


def test_underestimation_all_links_at_once():
    """The links' minima and "any negative" over (link, obstacle) pairs split
    G lanes per link, against the reference's link-by-link loop with its early
    return (whose minima are unused once a value is negative)."""
    rng = np.random.default_rng(5)
    for _ in range(400):
        L, n = int(rng.integers(1, 23)), int(rng.integers(0, 60))
        d = rng.normal(0.5, 0.4, size=(L, n)).astype(np.float32)
        maxd = np.float32(1000.0)
        # the reference: per link the min over obstacles, stop at the first negative
        neg_ref, mins_ref = False, []
        for i in range(L):
            m = maxd
            for j in range(n):
                if d[i, j] < 0:
                    neg_ref = True
                m = min_std(m, d[i, j])
            mins_ref.append(m)
            if neg_ref:
                break
        G = 32
        while G * L > 32:
            G //= 2
        part = np.full((L, G), maxd, np.float32)
        neg = False
        for i in range(L):
            for s in range(G):
                for j in range(s, n, G):
                    neg |= bool(d[i, j] < 0)
                    part[i, s] = min_std(part[i, s], d[i, j])
        mins = [np.float32(min(part[i])) for i in range(L)]
        assert neg == neg_ref
        if not neg:
            assert np.array(mins, np.float32).tobytes() == np.array(mins_ref, np.float32).tobytes()
