"""The bandpass median filter at windows above 1.  The reference fixes the
window at compile time (NMEDFILT, definitions.h:39, value 1: the identity)
and applies it in every bandpass correction (med_filter_bandpass,
median_filter.cpp:85-107); `hella_params.bp_median` makes it a runtime
window.  The flagger's bytes, bandpasses, statistics and time series must
equal the oracle's (whose median filter is pinned to the reference's own,
tests/test_golden.py) on the u8 path, the SCRUNCH path and the fp16 input
path, and a gulp loop's candidates must equal the oracle pipeline's."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline, small_params

pytestmark = pytest.mark.gpu


def _check(s, st_names, tr, ts, out, win_bytes):
    st = s.flag_stats(0)
    for k in st_names:
        assert np.array_equal(st[k].view(np.uint32), tr[k].view(np.uint32)), k
    for k in ("mean1", "std1", "mean2", "std2"):
        assert np.float32(st[k]).view(np.uint32) == np.float32(tr[k]).view(np.uint32), k
    assert np.array_equal(st["ts"].view(np.uint32), ts.view(np.uint32))
    assert np.array_equal(win_bytes, out)


@pytest.mark.parametrize("win,nchan", [(3, 256), (7, 160), (63, 128)])
def test_median_window_u8_path(hella, oracle, win, nchan):
    p = small_params(nchan=nchan, gulp=4096, bp_median=win)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=21 + win, rfi_chans=(3, 50), slope=0.4)
    s = hella.Search(hella.default_params(**p))
    x = sky.gulp(0, p["gulp"])
    x[:, 77] = 0
    s.load_gulp(x[None])
    s.fast_flagger()
    out, ts, tr = oracle.flag_beam(x, oracle.flag_params(bp_median=win))
    ref1, _, tr1 = oracle.flag_beam(x)
    assert not np.array_equal(tr["bp1"], tr1["bp1"])  # the window changes the bandpass
    _check(s, ("bp1", "bp2", "bp3"), tr, ts, out, s.copy_window(0)[-p["gulp"]:])


def test_median_window_scrunch_and_f16_paths(hella, oracle):
    entries = [(4, 2, 3.0, 1), (8, 4, 4.0, 1)]
    p = small_params(nchan=128, gulp=4096, bp_median=5)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=31, rfi_chans=(5, 90), slope=0.3,
                    spikes=[synth.Spike(1000, 3, 90.0)])
    x = sky.gulp(0, p["gulp"])
    s = hella.Search(hella.default_params(**p, scrunches=entries))
    s.load_gulp(x[None])
    s.fast_flagger()
    out, ts, tr = oracle.flag_beam(x, oracle.flag_params(scrunches=entries, bp_median=5))
    _check(s, ("bp1", "bp2", "bp3"), tr, ts, out, s.copy_window(0)[-p["gulp"]:])
    s.close()
    # an fp16 channel-major gulp with sub-integer detail (the DADA input)
    f = x.astype(np.float32) + np.random.default_rng(5).uniform(-0.45, 0.45, x.shape).astype(np.float32)
    ft = np.ascontiguousarray(f.astype(np.float16).T)
    s = hella.Search(hella.default_params(**p, input_format=1))
    s.load_gulp(ft[None])
    s.fast_flagger()
    out, ts, tr = oracle.flag_beam_f16(ft, oracle.flag_params(bp_median=5))
    _check(s, ("bp1", "bp2", "bp3"), tr, ts, out, s.copy_window(0)[-p["gulp"]:])


def test_median_window_gulp_loop_candidates(hella, oracle):
    params, sky = synth.config_plain(seed=11, nchan=128, gulp=2048, dm_max=300.0)
    params["bp_median"] = 9
    sky.bursts[0].amp *= 4
    s = hella.Search(hella.default_params(**params))
    pl = oracle_pipeline(oracle, params)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, params["gulp"])[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so and cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0
