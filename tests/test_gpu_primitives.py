"""The device decision trees on directed primitive cases (tests/golden/golden.npz
'adv_*', made by tests/golden/make_golden.py): degenerate and axis-parallel
segments, segments in face planes and along box edges, endpoints on faces,
edges and corners, clearances at the EQUALITY_THRESHOLD snap, and parallel,
collinear and degenerate segment pairs.  Each case goes through the same tree
instances the check kernels use (rpm_probe_primitives):

  * the reference's FP32 numerics are bit-equal to the answers of the
    reference's own CollisionAndDistance.cpp (adv_reference), except where
    that source reads its uninitialised edge matrix (adv_undefined), where they
    equal the oracle's documented "no edge" choice;
  * the FP64 form is bit-equal to the oracle's FP64 restatement (ref64);
  * the FP32 + FP64-recheck form equals FP64 on every collision case (0 flips)
    and is within 1e-5 m of it on every distance, both where the FP32 pass
    settles a case and where it hands it to the FP64 recheck.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
DIST_TOL_M = 1e-5   # the FP32 + recheck form's distance bound against FP64


def _same(a, b, dtype=np.float64):
    """Bit-equal, except that any NaN equals any NaN (the device and the host
    CPU write different NaN payloads; the reference only compares them)."""
    a, b = np.asarray(a, dtype), np.asarray(b, dtype)
    ib = np.uint64 if dtype == np.float64 else np.uint32
    return bool(np.all((np.isnan(a) & np.isnan(b)) | (a.view(ib) == b.view(ib))))


def _run(engine, precision, sel=None):
    import torch
    keys = ("adv_kind", "adv_A", "adv_B", "adv_X", "adv_r")
    arrs = [G[k] if sel is None else G[k][sel] for k in keys]
    kind, a, b, x, r = (torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in arrs)
    n = kind.shape[0]
    value = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    settled = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    engine.probe_primitives(precision, kind, a, b, x, r, value, settled)
    engine.sync()
    return value.cpu().numpy(), settled.cpu().numpy()


def test_fixture_covers_every_kind_and_the_undefined_branch():
    kind = G["adv_kind"]
    assert all((kind == k).sum() >= 1000 for k in (0, 1, 2))
    assert G["adv_undefined"].sum() > 0 and np.all(kind[G["adv_undefined"] == 1] == 1)
    assert np.isnan(G["adv_ref64"]).any()   # degenerate segment pairs reach the NaN-s path


def test_reference_numerics_equal_the_reference_source(engine):
    v, s = _run(engine, "fp32_ref")
    assert np.all(s == 1)
    # the reference's values are floats: compared as float32
    assert _same(v, G["adv_ref32"], np.float32)
    if "adv_reference" not in G:
        pytest.skip("fixture made without the reference tree")
    defined = G["adv_undefined"] == 0
    assert _same(v[defined], G["adv_reference"][defined], np.float32)


def test_fp64_form_equals_ref64(engine):
    v, _ = _run(engine, "fp64")
    assert _same(v, G["adv_ref64"])


def test_fp32_recheck_form_equals_fp64(engine):
    v, s = _run(engine, "fp32_recheck")
    kind, ref64 = G["adv_kind"], G["adv_ref64"]
    assert not np.any(s == 2), "the inlined and out-of-line collision trees disagree"
    assert set(np.unique(s)) <= {0, 1}
    coll = kind == 0
    # booleans: 0 flips against the FP64 form, settled or rechecked
    assert np.array_equal(v[coll], ref64[coll])
    # distances: within the bound where FP32 settled; bit-equal where FP64 rechecked
    for k in (1, 2):
        sel = kind == k
        both_nan = np.isnan(v[sel]) & np.isnan(ref64[sel])
        err = np.where(both_nan, 0.0, np.abs(v[sel] - ref64[sel]))
        assert not np.isnan(err).any()
        assert err.max() <= DIST_TOL_M, (k, err.max())
        re = sel & (s == 0)
        assert _same(v[re], ref64[re])
    # the directed cases sit on decision boundaries: many must go to the recheck
    assert (s == 0).sum() >= 50 and (s == 1).sum() >= 1000


def test_probe_rejects_missing_settled_output(engine):
    import torch
    from rpmplv2_gb300.engine import RpmError
    kind = torch.zeros(1, dtype=torch.int32, device="cuda")
    f = torch.zeros((1, 6), dtype=torch.float32, device="cuda")
    v = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(RpmError):
        engine.probe_primitives("fp32_recheck", kind, f, f, f, f[:, 0], v, None)
