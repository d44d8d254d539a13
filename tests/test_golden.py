"""The oracle against its committed golden fixtures (tests/golden/,
generated by tests/golden/make_golden.py): every routine of the path and
one whole step on a small even and a small odd grid.  Arrays must agree to
1e-13 of their largest magnitude, NaN canaries in the same places, integer
fields exactly; the logged residual sums (summed in a thread-count-dependent
order) to 1e-10."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

_SPEC = importlib.util.spec_from_file_location("make_golden", Path(__file__).parent / "golden" / "make_golden.py")
golden = importlib.util.module_from_spec(_SPEC)
_SPEC.loader.exec_module(golden)

LOOSE = {"do_tpls.err", "ls_iteration.err", "step.stats"}


@pytest.fixture(scope="module", params=list(golden.CASES))
def case(request):
    ref = np.load(golden.fixture_path(request.param))
    return request.param, {k: ref[k] for k in ref.files}, golden.compute(request.param)


def test_fixtures_cover_every_output(case):
    name, ref, got = case
    assert sorted(ref) == sorted(got)
    assert len(ref) >= 40


def test_oracle_reproduces_fixtures(case):
    name, ref, got = case
    bad = []
    for k, r in ref.items():
        g = np.asarray(got[k])
        assert g.shape == r.shape, k
        if r.dtype.kind in "iu":
            if not np.array_equal(g, r):
                bad.append((k, "integer mismatch"))
            continue
        nan_r, nan_g = np.isnan(r), np.isnan(g)
        if not np.array_equal(nan_r, nan_g):
            bad.append((k, "NaN pattern"))
            continue
        fr, fg = r[~nan_r], g[~nan_g]
        if fr.size == 0:
            continue
        scale = max(float(np.max(np.abs(fr))), 1e-300)
        err = float(np.max(np.abs(fg - fr))) / scale
        if err > (1e-10 if k in LOOSE else 1e-13):
            bad.append((k, err))
    assert not bad, (name, bad)


def test_fixtures_are_not_trivial(case):
    """The pinned fields carry the structure they should: an interface band,
    flow, a pressure gradient."""
    name, ref, _ = case
    assert np.count_nonzero(ref["status.istatus"]) > 0
    assert np.max(np.abs(ref["csf.fz"])) > 0
    assert np.max(np.abs(ref["step.U2"])) > 1.0
    assert np.ptp(ref["pressure.pres"][1:-1, 1:-1, 1:-1]) > 0
