"""CPU checks of the oracle: fp16 arithmetic, plan math, dedispersion
known-answer tests, statistics order, smoothing taps and the end-to-end
injection-recovery criterion of the reference (scripts/verify_injection_fil.py:30-40)."""
from fractions import Fraction

import numpy as np
import pytest

import synth
from helpers import oracle_pipeline, small_params


# ------------------------------------------------------------------- fp16

def test_h2f_all_patterns(oracle):
    L = oracle.lib()
    bits = np.arange(65536, dtype=np.uint16)
    ref = bits.view(np.float16).astype(np.float32)
    got = np.array([L.ho_h2f(int(b)) for b in bits], np.float32)
    fin = np.isfinite(ref)
    assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32))
    assert np.all(np.isnan(got[~fin]) == np.isnan(ref[~fin]))


def test_f2h_rounding(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(0)
    # all half midpoints and their neighbours, plus random floats over the range
    h = np.arange(0, 0x7bff, dtype=np.uint16).view(np.float16).astype(np.float32)
    mids = ((h[:-1].astype(np.float64) + h[1:]) / 2).astype(np.float32)
    x = np.concatenate([mids, np.nextafter(mids, 0), np.nextafter(mids, 1e9), h,
                        rng.uniform(-70000, 70000, 20000).astype(np.float32),
                        (rng.standard_normal(20000) * 1e-5).astype(np.float32)])
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    got = np.array([L.ho_f2h(float(v)) for v in x], np.uint16)
    assert np.array_equal(got, ref)


def _exact_round_half(q: Fraction) -> np.uint16:
    """Correctly rounded binary16 of a positive rational, by exact search."""
    lo, hi = 0, 0x7c00
    while hi - lo > 1:  # largest finite half <= q
        mid = (lo + hi) // 2
        if Fraction(float(np.uint16(mid).view(np.float16))) <= q:
            lo = mid
        else:
            hi = mid
    a = Fraction(float(np.uint16(lo).view(np.float16)))
    b = Fraction(float(np.uint16(lo + 1).view(np.float16))) if lo + 1 < 0x7c00 else Fraction(65520)
    if q - a < b - q or (q - a == b - q and lo % 2 == 0):
        return lo
    return lo + 1


def test_hdiv_correctly_rounded(oracle):
    L = oracle.lib()
    rng = np.random.default_rng(1)
    for _ in range(400):
        a, b = (int(v) for v in rng.integers(0x0400, 0x7000, 2))
        q = Fraction(float(np.uint16(a).view(np.float16))) / Fraction(float(np.uint16(b).view(np.float16)))
        if q >= 65504:
            continue
        assert L.ho_hdiv(a, b) == _exact_round_half(q)


# -------------------------------------------------------------- plan math

def test_dm_list_follows_tolerance(oracle):
    dt, f0, nchan = 1.048576e-3, 468.75, 512
    df = -(f0 - 375.0) / nchan
    dms = oracle.dm_list(0.0, 500.0, 500.0, 1.25, nchan, dt, f0, df)
    assert dms[0] == 0.0 and dms[-1] >= 500.0 and dms[-2] < 500.0
    assert np.all(np.diff(dms) > 0)
    # each step satisfies ts^2+ti^2+a^2 D'^2+b^2(D'-D)^2 = tol^2 (ts^2+ti^2+a^2 D^2)
    ts, ti, tol = dt * 1e6, 500.0, 1.25
    f = (f0 - (nchan / 2 - 0.5) * abs(df)) * 1e-3
    a = 8.3 * abs(df) / f**3
    b = a * nchan / 4
    D, Dn = dms[:-1].astype(np.float64), dms[1:].astype(np.float64)
    lhs = ts**2 + ti**2 + a**2 * Dn**2 + b**2 * (Dn - D) ** 2
    rhs = tol**2 * (ts**2 + ti**2 + a**2 * D**2)
    assert np.allclose(lhs, rhs, rtol=1e-4)  # trials are stored in fp32


def test_delays_monotone(oracle):
    nchan, dt, f0 = 256, 1e-3, 468.75
    df = -0.3
    tab = oracle.delay_table(nchan, dt, f0, df)
    assert tab[0] == 0 and np.all(np.diff(tab) > 0)
    # published cold-plasma delay of the bottom channel for DM 100
    f_lo = f0 + (nchan - 1) * df
    want = 4.148808e3 * 100 * (1 / f_lo**2 - 1 / f0**2) / dt
    assert abs(tab[-1] * 100 - want) < 1e-3 * want
    dms = oracle.dm_list(0.0, 300.0, 40.0, 1.3, nchan, dt, f0, df)
    d = oracle.dm_delays(dms, tab)
    assert np.all(np.diff(d, axis=0) >= 0) and np.all(np.diff(d, axis=1) >= 0)
    assert np.array_equal(d[:, 0], np.zeros(len(dms), np.int32))


# ------------------------------------------------------------ dedispersion

def _plan(oracle, nchan=64, dm_max=60.0):
    dt, f0 = 1e-3, 468.75
    df = -(f0 - 375.0) / nchan
    dms = oracle.dm_list(0.0, dm_max, 40.0, 1.3, nchan, dt, f0, df)
    return dms, oracle.dm_delays(dms, oracle.delay_table(nchan, dt, f0, df))


def test_dedisp_impulse(oracle):
    dms, delays = _plan(oracle)
    md = int(delays.max())
    nsamps = md + 300
    d = delays.shape[0] // 2
    x = np.zeros((nsamps, delays.shape[1]), np.uint8)
    t_true = 120
    for c in range(delays.shape[1]):  # a pulse dispersed exactly as trial d
        x[t_true + delays[d, c], c] = 1
    out = oracle.dedisperse(x, delays)
    assert out[d, t_true] == delays.shape[1]
    assert out[d].sum() == delays.shape[1]
    assert out.max() == out[d, t_true]


def test_dedisp_constant_and_killmask(oracle):
    dms, delays = _plan(oracle)
    nsamps = int(delays.max()) + 100
    x = np.full((nsamps, delays.shape[1]), 128, np.uint8)
    assert np.all(oracle.dedisperse(x, delays) == 128 * delays.shape[1])
    km = np.ones(delays.shape[1], np.int32)
    km[::3] = 0
    assert np.all(oracle.dedisperse(x, delays, killmask=km) == 128 * km.sum())


def test_dedisp_matches_numpy(oracle):
    dms, delays = _plan(oracle, nchan=48, dm_max=40.0)
    rng = np.random.default_rng(3)
    nsamps = int(delays.max()) + 257
    x = rng.integers(0, 256, (nsamps, delays.shape[1]), dtype=np.uint8)
    out = oracle.dedisperse(x, delays)
    nout = nsamps - int(delays.max())
    ref = np.zeros((len(dms), nout), np.int64)
    for d in range(len(dms)):
        for c in range(delays.shape[1]):
            ref[d] += x[delays[d, c]:delays[d, c] + nout, c]
    assert np.array_equal(out, ref.astype(np.float32))


def test_dedisp_properties(oracle):
    """Linearity (a + b with no byte overflow sums to the sum of the planes),
    a killmask equal to zeroing those channels, a time shift of the input
    shifting every trial, and DM trials in any order giving their rows."""
    dms, delays = _plan(oracle, nchan=64, dm_max=80.0)
    rng = np.random.default_rng(21)
    nsamps = int(delays.max()) + 400
    a = rng.integers(0, 128, (nsamps, 64), dtype=np.uint8)
    b = rng.integers(0, 128, (nsamps, 64), dtype=np.uint8)
    da, db, dab = (oracle.dedisperse(v, delays) for v in (a, b, a + b))
    assert np.array_equal(dab, da + db)
    km = (rng.random(64) > 0.3).astype(np.int32)
    zeroed = a * km[None, :].astype(np.uint8)
    assert np.array_equal(oracle.dedisperse(a, delays, killmask=km), oracle.dedisperse(zeroed, delays))
    k = 37
    shifted = np.concatenate([np.zeros((k, 64), np.uint8), a])[:nsamps]
    ds = oracle.dedisperse(shifted, delays)
    assert np.array_equal(ds[:, k:], da[:, :da.shape[1] - k])
    perm = rng.permutation(len(dms))
    dp = oracle.dedisperse(a, delays[perm], nout=da.shape[1])
    assert np.array_equal(dp, da[perm])


# -------------------------------------------------------------- statistics

def test_stddev_truncates_and_matches(oracle):
    rng = np.random.default_rng(4)
    x = rng.standard_normal((40, 700)).astype(np.float32) * 3 + 5
    x[:, 512:] = 1e6  # beyond 256*floor(700/256): ignored by the reference
    mean, sd = oracle.stddev_f32(x)
    ref = x[:, :512].astype(np.float64)
    assert abs(mean - ref.mean()) < 1e-5 * abs(ref.mean()) + 1e-6
    assert abs(sd - ref.std()) < 1e-5 * ref.std()


# -------------------------------------------------------------- smoothing

def test_smooth_taps(oracle):
    for sm in (1, 2, 8, 32):
        k = oracle.smooth_taps(sm)
        assert k.shape == (3, 2 * sm + 1)
        assert np.array_equal(k, k[:, ::-1])          # symmetric in time
        assert np.array_equal(k[0], k[2])             # DM weights 0.3 / 1 / 0.3
        assert abs(k.astype(np.float64).sum() - 1) < 1e-5
        assert np.argmax(k[1]) == sm


def test_smooth_constant_plane(oracle):
    L = oracle.lib()
    ndms, ntd, wmax, sm = 6, 600, 16, 4
    dd = np.full((ndms, ntd), 1000.0, np.float32)
    out = np.zeros((ndms - 2, 512), np.float32)
    L.ho_smooth_plane(dd.ctypes.data, ndms, ntd, ntd, sm, wmax, 0, out.ctypes.data, 512, 512)
    assert np.allclose(out, 1000.0, rtol=1e-5)


# -------------------------------------------------------------- flagger

def test_flagger_normalises_and_flags_rfi(oracle):
    rng = np.random.default_rng(5)
    w, nchan = 4096, 128
    x = np.clip(np.rint(rng.normal(128, 20, (w, nchan))), 0, 255).astype(np.uint8)
    x[:, 7] = 0  # a dead channel: its normalised mean is far below SPEC_MIN
    out, ts, tr = oracle.flag_beam(x)
    # requantised normal data: mean ~ 255/14*4, sd ~ 255/14
    assert abs(out.mean() - 72.9) < 2.0 and abs(out.std() - 18.2) < 2.0
    assert tr["bp2"][7] < -0.05                          # spectral flag (flagger.cu:151)
    others = np.delete(tr["bp2"], 7)
    assert np.all((others >= -0.05) & (others <= 0.15))
    assert tr["bp3"][7] == 1.0  # a flagged channel is set to 1 (flagger.cu:153)
    assert np.allclose(np.delete(tr["bp1"], 7), np.delete(x.mean(0), 7), rtol=1e-6)
    assert abs(ts.mean() - 1.0) < 0.02 and ts.std() < 0.15  # mean of ~N(1,1) over 128 channels


# ------------------------------------------------------- end to end (oracle)

def test_pipeline_recovers_injected_dm(oracle):
    params, sky = synth.config_plain(seed=11, nchan=128, gulp=4096, dm_max=400.0)
    sky.bursts[0].amp *= 2.0
    pl = oracle_pipeline(oracle, params)
    cands = None
    for g in range(pl.min_gulp + 1):
        cands, searched = pl.gulp_step(sky.gulp(g, params["gulp"])[None])
    assert searched and len(cands)
    best = cands[np.argmax(cands["snr"])]
    assert abs(pl.dms()[best["dm_idx"]] - sky.bursts[0].dm) < 2.0


def test_pipeline_ring_is_left_shift(oracle):
    """The overlap ring after gulp g's rewind holds the flagged stream
    samples [(g+2)G - NTIME, (g+1)G) at its start (casm_hella_refactored.cu:775-797)."""
    p = small_params()
    pl = oracle_pipeline(oracle, p)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=3)
    G, stream = p["gulp"], []
    for g in range(3):
        x = sky.gulp(g, G)
        stream.append(oracle.flag_beam(x)[0])
        pl.gulp_step(x[None])
    stream = np.concatenate(stream)
    ring = pl.ring(0)
    first = 4 * G - pl.ntime
    lo = max(0, -first)
    assert lo < pl.ntime - G
    assert np.array_equal(ring[lo:pl.ntime - G], stream[first + lo:3 * G])


def test_pipeline_killmask_drops_channels(oracle):
    """A beam's killmask leaves the dedispersed plane and candidates of a
    searched window exactly those of the same window with the killed channels
    zeroed, and leaves the other beam alone."""
    params, sky = synth.config_plain(seed=13, nchan=128, gulp=2048, dm_max=300.0)
    sky.bursts[0].amp *= 3
    params["nbeam"] = 2
    rng = np.random.default_rng(13)
    km = (rng.random(params["nchan"]) > 0.15).astype(np.int32)
    pk = oracle_pipeline(oracle, params)
    pk.set_killmask(1, km)
    p0 = oracle_pipeline(oracle, params)
    win = np.stack([oracle.flag_beam(sky.gulp(g, params["gulp"]))[0] for g in range(pk.min_gulp + 1)])
    win = win.reshape(-1, params["nchan"])[-pk.ntime:]
    zeroed = win * km[None, :].astype(np.uint8)
    a = pk.search_window(win, beam=1)
    b = p0.search_window(zeroed, beam=1)
    assert np.array_equal(a["dd"], b["dd"]) and len(a["cands"]) == len(b["cands"])
    assert np.array_equal(a["cands"], b["cands"])
    c = pk.search_window(win, beam=0)
    d = p0.search_window(win, beam=0)
    assert np.array_equal(c["dd"], d["dd"]) and np.array_equal(c["cands"], d["cands"])
    with pytest.raises(ValueError):
        pk.set_killmask(2, km)



def test_peak_gate_and_its_switch(oracle):
    """find_peaks searches only when the width-0 plane's deviation sigma0 lies
    in (0.1, 5) (peaks.cu:60, definitions.h:71-72); with the gate off
    (DEBUG_ALWAYS_FIND_PEAKS) it searches at SNR x sigma0 whatever sigma0."""
    rng = np.random.default_rng(3)
    boxes = (rng.standard_normal((2, 10, 512)) * 7.0).astype(np.float32)  # sigma0 about 7
    c, s0 = oracle.find_peaks(boxes, 2.0)
    assert s0 > 5 and len(c) == 0
    c, s0 = oracle.find_peaks(boxes, 2.0, gate=False)
    assert len(c) > 0 and np.all(c["snr"] > 2.0 * np.float32(s0))
