"""This library's smoothing FIR and SCRUNCH box filter against the filters
the reference actually runs: NPP's nppiFilterBorder_32f_C1R (smoothing,
src/hella/src/smooth.cpp:21-127) and nppiFilterBorder32f_16f_C1R (box,
src/hella/src/convolution.cu:20-55), called on the GPU through
oracle/npp_ref.py (test infrastructure; the product never links NPP).

NPP's summation order is closed, so neither filter can be reproduced bit
for bit; the smoothing is held to it within RTOL on the smoothed planes
(and that tolerance carried through the normalisation), with the candidate
lists (width, DM index, sample) required identical.  The reference's own
statistics, normalisation and peak finding (the oracle, pinned to the
reference's code by test_golden.py) run on NPP's planes."""
import numpy as np
import pytest

import synth
from helpers import oracle_pipeline, small_params

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # smoothed planes, relative; normalised values carry RTOL * (|x| + |mean|) / std


@pytest.fixture(scope="module")
def npp():
    import npp_ref

    npp_ref.lib()
    return npp_ref


def _searched(hella, oracle, params, sky):
    """Runs the GPU search to its first searched gulp; checks the GPU's
    standardised planes against the oracle on the same window."""
    s = hella.Search(hella.default_params(**params))
    pl = oracle_pipeline(oracle, params)
    G = params["gulp"]
    for g in range(pl.min_gulp + 1):
        x = sky.gulp(g, G)[None]
        if g == pl.min_gulp:
            s.clear_peaks()
            s.load_gulp(x)
            s.fast_flagger()
            win = s.copy_window(0)
            s.dedisperse(0)
            s.smooth(1)
            s.find_peaks(0)
        else:
            s.process_gulp(x)
    ref = pl.search_window(win, 0)
    boxes = s.copy_boxes()
    assert np.array_equal(boxes.view(np.uint32), ref["boxes"].view(np.uint32))
    mean, std, s0 = s.smooth_stats()
    out = dict(dd=s.copy_dedisp(), boxes=boxes, mean=mean, std=std, sigma0=s0, cands=s.get_peaks(),
               ntime_out=s.info.ntime_out)
    s.close()
    return out


def _reference_smoothing(oracle, npp, dd, wmin, wmax, ntime_out, snr):
    """smooth(p, 1) + find_peaks with NPP's filter and the reference's
    statistics, normalisation (AddC(-mean), MulC(1/std)) and peak finding."""
    sms = []
    sm = wmin
    while sm < wmax:
        sms.append(sm)
        sm *= 2
    pre = npp.smooth_planes(dd, [oracle.smooth_taps(sm) for sm in sms], wmax, ntime_out)
    norm = pre.copy()
    mean, std = np.zeros(len(sms), np.float32), np.zeros(len(sms), np.float32)
    for b in range(len(sms)):
        m, s = oracle.stddev_f32(pre[b])
        mean[b], std[b] = m, s
        if s > 0:
            norm[b] = (pre[b] + np.float32(-1.0 * np.float32(m))) * (np.float32(1.0) / np.float32(s))
    cands, s0 = oracle.find_peaks(norm, snr)
    return sms, pre, norm, mean, std, cands, s0


def _check(oracle, npp, params, got):
    wmin, wmax = params["width_min"], params["width_max"]
    sms, pre, norm, mean, std, cands, s0 = _reference_smoothing(oracle, npp, got["dd"], wmin, wmax,
                                                                got["ntime_out"], params["snr"])
    worst = 0.0
    for b, sm in enumerate(sms):
        mine = oracle.smooth_plane(got["dd"], sm, wmax, got["ntime_out"])  # the GPU's planes, bit for bit
        rel = float(np.max(np.abs(mine.astype(np.float64) - pre[b]) / np.abs(pre[b])))
        worst = max(worst, rel)
        assert rel <= RTOL, (sm, rel)
    assert np.all(np.abs(got["mean"] - mean) <= RTOL * np.abs(mean))
    assert np.all(np.abs(got["std"] - std) <= RTOL * (np.abs(mean) + std))
    m, s = mean[:, None, None], std[:, None, None]
    tol = RTOL * ((np.abs(pre) + np.abs(m)) + np.abs(norm) * (np.abs(m) + s)) / s
    assert np.all(np.abs(got["boxes"] - norm) <= tol)
    c = got["cands"]
    assert len(c) == len(cands)
    for k in ("width", "dm_idx", "samp"):
        assert np.array_equal(c[k], cands[k]), k
    w = cands["width"]
    ctol = RTOL * ((np.abs(cands["snr"]) * std[w] + 2 * np.abs(mean[w])) + np.abs(cands["snr"]) *
                   (np.abs(mean[w]) + std[w])) / std[w]
    assert np.all(np.abs(c["snr"] - cands["snr"]) <= ctol)
    assert abs(got["sigma0"] - s0) <= RTOL * (abs(mean[0]) + std[0]) / std[0]
    return worst, len(c), int(np.sum(c["snr"].view(np.uint32) != cands["snr"].view(np.uint32)))


def test_plain_config_smoothing_matches_npp(hella, oracle, npp):
    """512 channels, gulp 16384, DM 0-500, widths 1..32: NPP's planes, the
    statistics, standardised planes and candidates."""
    params, sky = synth.config_plain(seed=1)
    got = _searched(hella, oracle, params, sky)
    worst, n, snr_bits = _check(oracle, npp, params, got)
    assert n > 0
    print(f"plain: planes within {worst:.2e} of NPP; {n} candidates identical, {snr_bits} S/N differ in low bits")


@pytest.mark.parametrize("wmin,wmax", [(1, 16), (3, 400), (1, 2048), (5, 11)])
def test_smoothing_width_sets_match_npp(hella, oracle, npp, wmin, wmax):
    p = small_params(nchan=128, gulp=4096, dm_max=60.0, width_min=wmin, width_max=wmax, snr=5.0)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=31 + wmin, rfi_chans=(9,), slope=0.2)
    got = _searched(hella, oracle, p, sky)
    worst, n, snr_bits = _check(oracle, npp, p, got)
    print(f"widths {wmin}-{wmax}: planes within {worst:.2e} of NPP; {n} candidates identical")


@pytest.mark.parametrize("xw,yw", [(4, 4), (16, 2), (8, 8), (3, 5)])
def test_scrunch_box_filter_against_npp(oracle, npp, xw, yw):
    """The box filter of the SCRUNCH branch on standardised data and on 0/1
    masks (apply_scrunch, flagger.cu:302-334).  fp32 sums rounded to fp16:
    the orders differ only where a sum lies within an fp32 rounding of an
    fp16 rounding boundary, so results agree to one fp16 unit (+0 and -0
    count as equal), a mask's box is non-zero at the same places (the
    replace_data decision), and a box of a power-of-two area on a mask is
    exact in any order."""
    rng = np.random.default_rng(xw * 31 + yw)
    k = float(np.float32(1.0 / xw / yw))
    data = rng.standard_normal((256, 2048)).astype(np.float16).view(np.uint16)
    mask = (rng.random((256, 2048)) < 0.02).astype(np.float16).view(np.uint16)
    for name, x in (("data", data), ("mask", mask)):
        a = npp.box_filter_f16(x, xw, yw, k)
        o = oracle.box_filter(x, xw, yw, k)
        fa, fo = a.view(np.float16).astype(np.float32), o.view(np.float16).astype(np.float32)
        same = (a == o) | ((fa == 0) & (fo == 0))
        diff = np.abs(a.astype(np.int32) - o.astype(np.int32))
        assert np.all(same | (diff <= 1)), name
        assert np.mean(~same) < 0.01, (name, np.mean(~same))
        if name == "mask":
            assert np.array_equal(fa > 0, fo > 0)
            if (xw * yw) & (xw * yw - 1) == 0:
                assert np.all(same)
        print(f"box {xw}x{yw} {name}: {int(np.sum(~same))} of {a.size} differ by one fp16 unit")
