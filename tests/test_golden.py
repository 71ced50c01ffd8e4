"""The oracle against golden outputs of the reference's own code.

tests/golden/reference_fixtures.json holds what the reference's flagger
(fast_flagger, with and without SCRUNCH entries), calculate_stddev<float>
and <half>, median_filter, smooth (taps and standardised planes) and
find_peaks produced on seeded inputs (tests/golden/cases.py), run on the
CPU by tests/golden/make_golden.py.  The oracle must reproduce every byte
and every float bit.

The reference's smoothing FIR is NPP's (closed); the fixtures ran it through
a stand-in that applies the 3 x (2sm+1) kernel tap by tap.  The oracle's
direct form reproduces that bit for bit (taps, anchor, crop, statistics,
normalisation and peak order are pinned); the factored form the GPU
computes is held to it within the tolerance below, and to NPP itself by
tests/test_gpu_npp.py."""
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
    boxes, _, _ = oracle.smooth_normalise(cases.smooth_input(c), c["wmin"], c["wmax"], c["ntime_out"], anchor=1,
                                          direct=True)
    assert cases.sha(boxes) == want["boxes_sha"]
    cands, _ = oracle.find_peaks(boxes, c["snr"])
    assert len(cands) == want["npeaks"] > 0
    arr = np.stack([cands["snr"].view(np.int32), cands["width"], cands["dm_idx"], cands["samp"]])
    assert cases.sha(arr.astype(np.int32)) == want["peaks_sha"]


# Relative tolerance of smoothed (pre-normalisation) planes against the
# reference's filter.  Normalisation subtracts a mean that is large against
# the std, so a normalised value carries it as RTOL * (|x| + |mean|) / std.
RTOL = 1e-5


@pytest.mark.parametrize("i", range(len(cases.SMOOTH_CASES)))
def test_factored_smoothing_against_direct_kernel(oracle, i):
    """The factored FIR (0.3 * (row above + row below) + row, then the
    middle-row taps) against the kernel applied tap by tap: planes within
    RTOL, the same candidates (width, DM, sample) in the same order, S/N
    within the tolerance carried through the normalisation."""
    c = cases.SMOOTH_CASES[i]
    dd = cases.smooth_input(c)
    worst = 0.0
    for b in range(16):
        sm = c["wmin"] << b
        if sm >= c["wmax"]:
            break
        f = oracle.smooth_plane(dd, sm, c["wmax"], c["ntime_out"])
        d = oracle.smooth_plane(dd, sm, c["wmax"], c["ntime_out"], direct=True)
        rel = float(np.max(np.abs(f.astype(np.float64) - d) / np.abs(d)))
        worst = max(worst, rel)
        assert rel <= RTOL, (sm, rel)
    assert worst > 0  # the two forms round differently: the check is not vacuous
    bf, mf, sf = oracle.smooth_normalise(dd, c["wmin"], c["wmax"], c["ntime_out"])
    bd, md, sd = oracle.smooth_normalise(dd, c["wmin"], c["wmax"], c["ntime_out"], direct=True)
    # a plane error of RTOL * |x| moves the mean by as much and the std by RTOL * (|mean| + std) at most
    assert np.all(np.abs(mf - md) <= RTOL * np.abs(md))
    assert np.all(np.abs(sf - sd) <= RTOL * (np.abs(md) + sd))
    cf, _ = oracle.find_peaks(bf, c["snr"])
    cd, _ = oracle.find_peaks(bd, c["snr"])
    for k in ("width", "dm_idx", "samp"):
        assert np.array_equal(cf[k], cd[k]), k
    tol = RTOL * (np.abs(cd["snr"]) * sd[cd["width"]] + 2 * np.abs(md[cd["width"]])) / sd[cd["width"]]
    assert np.all(np.abs(cf["snr"] - cd["snr"]) <= tol)
