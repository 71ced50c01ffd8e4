"""The oracle against golden outputs of the reference's own code.

tests/golden/reference_fixtures.json holds what the reference's flagger
(fast_flagger, with and without SCRUNCH entries), calculate_stddev<float>
and <half>, median_filter, smooth (taps and standardised planes) and
find_peaks produced on seeded inputs (tests/golden/cases.py), run on the
CPU by tests/golden/make_golden.py.  The oracle must reproduce every byte
and every float bit."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = json.loads((GOLDEN / "reference_fixtures.json").read_text())

import golden.cases as cases  # noqa: E402


@pytest.mark.parametrize("c", cases.FLAG_CASES, ids=[c["name"] for c in cases.FLAG_CASES])
def test_flagger_matches_reference(oracle, c):
    want = next(f for f in FIX["flag"] if f["name"] == c["name"])
    x = cases.flag_input(c)
    fp = oracle.flag_params(-0.05, 0.15, c.get("flag1", -1), c.get("flag2", -1), c["scrunch"])
    fs = np.zeros(cases.NCHAN, np.float32)
    out, ts, _ = oracle.flag_beam(x, fp, flagspec=fs)
    assert cases.bits(ts[:16]) == want["ts_head"]
    assert cases.sha(ts) == want["ts_sha"]
    assert cases.bits(fs) == want["flagspec"]
    assert cases.sha(out) == want["out_sha"], f"mean {out.mean()} vs {want['out_mean']}"


@pytest.mark.parametrize("i", range(len(cases.STAT_CASES)))
def test_stddev_matches_reference(oracle, i):
    c = cases.STAT_CASES[i]
    L = oracle.lib()
    for key, x, fn in (("stddev_f32", cases.stat_input_f32(c), L.ho_stddev_f32),
                       ("stddev_f16", cases.stat_input_f16(c), L.ho_stddev_f16)):
        want = FIX[key][i]
        m = np.zeros(1, np.float32)
        s = fn(x.ctypes.data, c["w"], c["h"], c["stride"], m.ctypes.data)
        assert cases.bits(m)[0] == want["mean"], key
        assert cases.bits([s])[0] == want["std"], key


@pytest.mark.parametrize("i", range(len(cases.MEDIAN_CASES)))
def test_median_filter_matches_reference(oracle, i):
    c = cases.MEDIAN_CASES[i]
    want = FIX["median"][i]
    out, mn = oracle.median_filter(cases.median_input(c), c["window"])
    assert cases.sha(out) == want["out_sha"]
    assert cases.bits([mn])[0] == want["mean"]


@pytest.mark.parametrize("i", range(len(cases.SMOOTH_CASES)))
def test_smooth_and_peaks_match_reference(oracle, i):
    c = cases.SMOOTH_CASES[i]
    want = FIX["smooth"][i]
    nbox = len(want["taps"]) and sum(1 for b in range(16) if (c["wmin"] << b) < c["wmax"])
    taps = np.concatenate([oracle.smooth_taps(c["wmin"] << b).ravel() for b in range(nbox)])
    assert cases.bits(taps) == want["taps"]
    boxes, _, _ = oracle.smooth_normalise(cases.smooth_input(c), c["wmin"], c["wmax"], c["ntime_out"], anchor=1)
    assert cases.sha(boxes) == want["boxes_sha"]
    cands, _ = oracle.find_peaks(boxes, c["snr"])
    assert len(cands) == want["npeaks"] > 0
    arr = np.stack([cands["snr"].view(np.int32), cands["width"], cands["dm_idx"], cands["samp"]])
    assert cases.sha(arr.astype(np.int32)) == want["peaks_sha"]
