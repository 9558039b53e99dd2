"""The serving latency summary (serve.latency_summary) that the bench's serve
line reports: which requests form the 2,048-8,192 bucket, the percentiles in
milliseconds, the per-kind split and the DRGBT kinds kept apart.  CPU only,
on synthetic timing records."""
from types import SimpleNamespace

import numpy as np

from rpmplv2_gb300 import serve
from rpmplv2_gb300._abi import RPM_ERR_ADMISSION


def _t(submit, launch, done, status=0, batch=1):
    return SimpleNamespace(t_submit=submit, t_launch=launch, t_done=done, status=status, batch_size=batch)


def test_bucket_percentiles_and_kinds():
    rng = np.random.default_rng(2)
    timings, meta = [], []
    kinds = ["valid", "distance", "edges", "reached", "motion"]
    for i in range(2000):
        kind = kinds[i % 5]
        size = int(rng.integers(1, 65537))
        t0 = i * 1e-4
        lat = float(rng.uniform(1e-4, 2e-3))
        status = RPM_ERR_ADMISSION if i % 97 == 0 else 0
        timings.append(_t(t0, t0 + lat / 3, t0 + lat, status, batch=int(rng.integers(1, 5))))
        meta.append((kind, size, size, 0))
    s = serve.latency_summary(timings, meta)
    lat_ms = np.array([(t.t_done - t.t_submit) * 1e3 for t in timings])
    ok = np.array([t.status == 0 for t in timings])
    k = np.array([m[0] for m in meta])
    sz = np.array([m[1] for m in meta])
    checks = np.isin(k, ["valid", "distance", "edges"])
    sel = ok & checks & (sz >= 2048) & (sz <= 8192)
    assert s["requests"] == 2000 and s["completed"] == int(ok.sum())
    assert s["rejected"] == int((~ok).sum())
    assert np.isclose(s["p99_ms_4096"], np.percentile(lat_ms[sel], 99))
    assert np.isclose(s["p50_ms_4096"], np.percentile(lat_ms[sel], 50))
    assert np.isclose(s["p99_ms_4096_configs"], np.percentile(lat_ms[sel & (k != "edges")], 99))
    for kind in ("valid", "distance", "edges"):
        m = sel & (k == kind)
        assert s["bucket_4096_by_kind"][kind]["requests"] == int(m.sum())
        assert np.isclose(s["bucket_4096_by_kind"][kind]["p99_ms"], np.percentile(lat_ms[m], 99))
    # the DRGBT kinds are outside the size buckets, reported apart
    assert s["drgbt_horizon"]["requests"] == int((ok & (k == "reached")).sum())
    assert s["motion_validity"]["requests"] == int((ok & (k == "motion")).sum())
    assert np.isclose(s["p99_ms_le4096"], np.percentile(lat_ms[ok & checks & (sz <= 4096)], 99))


def test_empty_bucket_reports_none():
    timings = [_t(0.0, 0.0001, 0.001)]
    meta = [("valid", 100, 100, 0)]
    s = serve.latency_summary(timings, meta)
    assert s["p99_ms_4096"] is None and s["completed"] == 1
