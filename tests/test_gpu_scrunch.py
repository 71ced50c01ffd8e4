"""SCRUNCH flagging (apply_scrunch with flag = 1, flagger.cu:271-343) on the
GPU: ring bytes, flagger statistics, time series and the accumulated
per-channel flag fractions bit-exact against the oracle, which is pinned to
the reference's own flagger code (tests/golden)."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline, small_params

pytestmark = pytest.mark.gpu

SCR = [(4, 2, 3.0, 1), (8, 4, 4.0, 1), (16, 1, 3.5, 1)]


@pytest.mark.parametrize("entries,flags", [(SCR[:1], (-1, -1)), (SCR, (10, 20))])
def test_scrunch_flagger_bit_exact(hella, oracle, entries, flags):
    p = small_params(nchan=128, gulp=4096)
    p.update(flag1=flags[0], flag2=flags[1])
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=31, rfi_chans=(5, 90), slope=0.3,
                    spikes=[synth.Spike(1000, 3, 90.0), synth.Spike(3000, 8, 60.0)])
    s = hella.Search(hella.default_params(**p, scrunches=entries))
    fspec = np.zeros(p["nchan"], np.float32)
    fp = oracle.flag_params(flag1=flags[0], flag2=flags[1], scrunches=entries)
    for g in range(2):
        x = sky.gulp(g, p["gulp"])
        x[:, 77] = 0
        s.load_gulp(x[None])
        s.fast_flagger()
        out, ts, tr = oracle.flag_beam(x, fp, fspec)
        st = s.flag_stats(0)
        for k in ("bp1", "bp2", "bp3"):
            assert np.array_equal(st[k].view(np.uint32), tr[k].view(np.uint32)), (g, k)
        for k in ("mean1", "std1", "mean2", "std2"):
            assert np.float32(st[k]).view(np.uint32) == np.float32(tr[k]).view(np.uint32), (g, k)
        assert np.array_equal(st["ts"].view(np.uint32), ts.view(np.uint32))
        assert np.array_equal(s.copy_window(0)[-p["gulp"]:], out), g
        assert np.array_equal(s.flag_spec().view(np.uint32), fspec.view(np.uint32)), g
        s.rewind()
    assert fspec.max() > 0


@pytest.mark.parametrize("add_mode", [None, 6])
def test_scrunch_gulp_loop_and_batch(hella, oracle, add_mode):
    """add_mode 6: both contexts dedisperse through quad rows."""
    params, _ = synth.config_plain(seed=33, nchan=128, gulp=2048, dm_max=400.0)
    skies = [synth.config_plain(seed=34 + b, nchan=128, gulp=2048, dm_max=400.0)[1] for b in range(2)]
    for sk in skies:
        sk.bursts[0].amp *= 3
    s = hella.Search(hella.default_params(**dict(params, nbeam=2), scrunches=SCR[:2]))
    pl = oracle_pipeline(oracle, params, nbeam=2, scrunches=SCR[:2])
    bt = hella.Batch(hella.default_params(**dict(params, nbeam=2), scrunches=SCR[:2]))
    if add_mode:
        s.set_tuning(hella.HellaTuning(16, 4, 16, 0, 4, add_mode))
        bt.set_tuning(hella.HellaTuning(16, 4, 16, 0, 4, add_mode))
    # flag statistics fed from the device's cumulative flag spectrum each gulp
    # (casm_hella_refactored.cu:708-716), counted like the host model below
    ntime = s.info.ntime
    fs = hella.FlagStats(params["nchan"], ntime)
    prev, want_counts = np.zeros(params["nchan"], np.float32), np.zeros(params["nchan"], np.int64)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        got, _ = s.process_gulp(x)
        want, _ = pl.gulp_step(x)
        assert cands_equal(got, want), g
        bgot, counts, _ = bt.process_gulp(x)
        assert cands_equal(bgot, want), g
        cum = s.flag_spec()
        fs.update(cum)
        ref = pl.flagspec()
        want_counts += (ntime * (ref - prev).astype(np.float64)).astype(np.int64)  # fp32 difference, as in C
        prev = ref.copy()
        total += len(got)
    assert total > 0
    assert np.array_equal(fs.counts(), want_counts)
    assert np.array_equal(s.flag_spec().view(np.uint32), pl.flagspec().view(np.uint32))
    assert np.array_equal(bt.flag_spec().view(np.uint32), pl.flagspec().view(np.uint32))
