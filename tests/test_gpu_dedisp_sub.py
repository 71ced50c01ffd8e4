"""Add mode 4 of the dedispersion kernel: four-channel sums built once per
relative-delay pattern of a 16-trial tile and shared by the tile's trials.
Integer sums in any grouping are the same numbers, so every plane must be
bit-exact against the oracle's channel-by-channel sums and against the
other add modes: channel counts that are not multiples of four (killmasks),
partial last tiles, the full single beam, and the batched context with
per-beam killmasks."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline

pytestmark = pytest.mark.gpu

MODE4 = (0, 4, 8, 0, 8, 4)  # dm_per_block, samples, chan_chunk, stages, group, add_mode


def _window_dedisp(hella, oracle, params, sky, killmask=None):
    s = hella.Search(hella.default_params(**params))
    if killmask is not None:
        s.set_killmask(killmask)
    info = s.info
    for g in range(info.min_gulp + 1):
        s.clear_peaks()
        s.load_gulp(sky.gulp(g, params["gulp"])[None])
        s.fast_flagger()
        if g < info.min_gulp:
            s.rewind()
    win = s.copy_window(0)
    s.set_tuning(hella.HellaTuning(*MODE4))
    s.dedisperse(0)
    got = s.copy_dedisp()
    dmsl = s.dm_list()
    f32 = lambda v: float(np.float32(v))
    delays = oracle.dm_delays(dmsl, oracle.delay_table(params["nchan"], f32(params["plan_dt"]),
                                                       f32(params["f0_mhz"]), f32(params["df_mhz"])))
    want = oracle.dedisperse(win, delays, killmask=killmask, nout=s.info.ntime_dd)
    s.set_tuning(hella.HellaTuning(0, 4, 8, 0, 8, 0))
    s.dedisperse(0)
    other = s.copy_dedisp()
    s.close()
    return got, want, other


@pytest.mark.parametrize("nchan,dm_max,kill", [(128, 400.0, 0), (160, 300.0, 1), (256, 1000.0, 2), (96, 60.0, 3)])
def test_sub_band_planes_exact(hella, oracle, nchan, dm_max, kill):
    params, sky = synth.config_plain(seed=20 + kill, nchan=nchan, gulp=2048, dm_max=dm_max)
    km = None
    rng = np.random.default_rng(kill)
    if kill == 1:  # 17 killed channels: 143 active, the last group of three
        km = np.ones(nchan, np.int32)
        km[rng.choice(nchan, 17, replace=False)] = 0
    elif kill == 2:  # runs and single channels, 2 left over in the last group
        km = (rng.random(nchan) > 0.1).astype(np.int32)
        km[40:57] = 0
        while int(km.sum()) % 4 != 2:
            km[int(rng.integers(0, nchan))] = 0
    elif kill == 3:  # a single active channel
        km = np.zeros(nchan, np.int32)
        km[33] = 1
    got, want, other = _window_dedisp(hella, oracle, params, sky, km)
    assert np.array_equal(got, want)
    assert np.array_equal(got, other)


def test_sub_band_gulp_loop_candidates(hella, oracle):
    params, sky = synth.config_plain(seed=14, nchan=160, gulp=2048, dm_max=300.0)
    sky.bursts[0].amp *= 4
    km = (np.random.default_rng(14).random(params["nchan"]) > 0.15).astype(np.int32)
    s = hella.Search(hella.default_params(**params))
    s.set_killmask(km)
    s.set_tuning(hella.HellaTuning(*MODE4))
    pl = oracle_pipeline(oracle, params)
    pl.set_killmask(0, km)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, params["gulp"])[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so and cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0


def test_sub_band_full_beam(hella):
    """The full single beam (2048 channels, 2501 trials, spreads up to 872
    samples): the whole dedispersed plane identical to add mode 2's."""
    params, sky = synth.config_full(seed=2)
    s = hella.Search(hella.default_params(**params))
    for g in range(s.info.min_gulp + 1):
        s.clear_peaks()
        s.load_gulp(sky.gulp(g, params["gulp"])[None])
        s.fast_flagger()
        if g < s.info.min_gulp:
            s.rewind()
    s.set_tuning(hella.HellaTuning(0, 4, 8, 0, 8, 2))
    s.dedisperse(0)
    ref = s.copy_dedisp()
    s.set_tuning(hella.HellaTuning(*MODE4))
    s.dedisperse(0)
    assert np.array_equal(s.copy_dedisp(), ref)
    ms4 = s.time_dedisp(hella.HellaTuning(*MODE4), 3)
    ms2 = s.time_dedisp(hella.HellaTuning(0, 4, 8, 0, 8, 2), 3)
    print(f"full beam dedispersion: add mode 4 {ms4:.2f} ms, add mode 2 {ms2:.2f} ms")
    s.close()


def test_sub_band_batch_killmasks(hella):
    """The batched context in add mode 4 (the plan's tables for every beam,
    killed channels packed as zeros) against single-beam contexts."""
    params, _ = synth.config_plain(seed=40, nchan=128, gulp=2048, dm_max=400.0)
    nb = 5
    rng = np.random.default_rng(41)
    ceilings = np.array([400.0, 250.0, 330.0, 180.0, 400.0], np.float32)
    kill = (rng.random((nb, 128)) > rng.uniform(0, 0.1, (nb, 1))).astype(np.int32)
    kill[1] = 0
    kill[1, 77] = 1
    kill[3, :9] = 0
    skies = []
    for b in range(nb):
        sk = synth.config_plain(seed=42 + b, nchan=128, gulp=2048, dm_max=float(ceilings[b]))[1]
        sk.bursts[0].amp *= 3
        skies.append(sk)
    bt = hella.Batch(hella.default_params(**dict(params, nbeam=nb)), dm_max=ceilings, killmask=kill)
    bt.set_tuning(hella.HellaTuning(*MODE4))
    singles = []
    for b in range(nb):
        s = hella.Search(hella.default_params(**dict(params, dm_max=float(ceilings[b]), beam0=b, nbeam=1)))
        s.set_killmask(kill[b])
        singles.append(s)
    total = 0
    for g in range(max(s.info.min_gulp for s in singles) + 2):
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        got, counts, searched = bt.process_gulp(x)
        off = 0
        for b, s in enumerate(singles):
            want, sw = s.process_gulp(x[b:b + 1])
            mine = got[off:off + counts[b]]
            off += counts[b]
            assert searched[b] == sw and cands_equal(mine, want), (g, b)
            if sw:
                assert np.array_equal(bt.copy_dedisp(b), s.copy_dedisp()), (g, b)
            total += len(want)
    assert total > 0
