"""Add modes 5 and 6 of the dedispersion: rows of channel pairs / quads.
Adjacent active channels are summed once per window and pattern of
relative delays into rows in HBM, and each 16-trial tile sums the rows of
its trials' patterns.  Integer sums
in any grouping are the same numbers, so every plane must be bit-exact
against the oracle's channel-by-channel sums and against the other add
modes: odd active-channel counts (the last channel alone), pairs of
non-adjacent active channels, a single active channel, both stage widths,
the ring's window wrapping over gulps, the full single beam, and the
tuner choosing among all modes."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline

pytestmark = pytest.mark.gpu

MODE5 = (0, 4, 8, 0, 8, 5)     # dm_per_block, samples, chan_chunk, stages, group, add_mode
MODE5_16 = (16, 4, 16, 0, 8, 5)
MODE6 = (16, 4, 16, 0, 8, 6)     # rows of four channels
MODE6_8 = (0, 4, 8, 0, 8, 6)


def _window(hella, params, sky, killmask=None, gulps=None):
    s = hella.Search(hella.default_params(**params))
    if killmask is not None:
        s.set_killmask(killmask)
    n = s.info.min_gulp + 1 if gulps is None else gulps
    for g in range(n):
        s.clear_peaks()
        s.load_gulp(sky.gulp(g, params["gulp"])[None])
        s.fast_flagger()
        if g < n - 1:
            s.rewind()
    return s


def _oracle_plane(oracle, params, s, win, killmask):
    f32 = lambda v: float(np.float32(v))
    delays = oracle.dm_delays(s.dm_list(), oracle.delay_table(params["nchan"], f32(params["plan_dt"]),
                                                              f32(params["f0_mhz"]), f32(params["df_mhz"])))
    return oracle.dedisperse(win, delays, killmask=killmask, nout=s.info.ntime_dd)


@pytest.mark.parametrize("shape", [MODE5, MODE5_16, MODE6, MODE6_8])
@pytest.mark.parametrize("nchan,dm_max,kill", [(128, 400.0, 0), (160, 300.0, 1), (256, 1000.0, 2), (96, 60.0, 3),
                                               (64, 800.0, 4)])
def test_pair_rows_planes_exact(hella, oracle, nchan, dm_max, kill, shape):
    params, sky = synth.config_plain(seed=50 + kill, nchan=nchan, gulp=2048, dm_max=dm_max)
    km = None
    rng = np.random.default_rng(kill)
    if kill == 1:  # 17 killed channels: 143 active, the last one alone
        km = np.ones(nchan, np.int32)
        km[rng.choice(nchan, 17, replace=False)] = 0
    elif kill == 2:  # runs and single channels: pairs of channels far apart, an odd count
        km = (rng.random(nchan) > 0.1).astype(np.int32)
        km[40:57] = 0
        while int(km.sum()) % 2 != 1:
            km[int(rng.integers(0, nchan))] = 0
    elif kill == 3:  # a single active channel
        km = np.zeros(nchan, np.int32)
        km[33] = 1
    elif kill == 4:  # every other channel killed: every pair spans a killed one
        km = np.zeros(nchan, np.int32)
        km[::2] = 1
    s = _window(hella, params, sky, km)
    win = s.copy_window(0)
    s.set_tuning(hella.HellaTuning(*shape))
    s.dedisperse(0)
    got = s.copy_dedisp()
    want = _oracle_plane(oracle, params, s, win, km)
    assert np.array_equal(got, want)
    s.set_tuning(hella.HellaTuning(0, 4, 8, 0, 8, 0))
    s.dedisperse(0)
    assert np.array_equal(s.copy_dedisp(), got)
    s.close()


@pytest.mark.parametrize("shape", [MODE5, MODE6])
def test_pair_rows_window_wraps(hella, oracle, shape):
    """Windows that start anywhere in the ring (gulps 3..6 of a ring of
    about two gulps): every window's plane exact."""
    params, sky = synth.config_plain(seed=61, nchan=96, gulp=1024, dm_max=200.0)
    s = hella.Search(hella.default_params(**params))
    s.set_tuning(hella.HellaTuning(*shape))
    checked = 0
    for g in range(s.info.min_gulp + 5):
        s.clear_peaks()
        s.load_gulp(sky.gulp(g, params["gulp"])[None])
        s.fast_flagger()
        if g >= s.info.min_gulp:
            win = s.copy_window(0)
            s.dedisperse(0)
            assert np.array_equal(s.copy_dedisp(), _oracle_plane(oracle, params, s, win, None)), g
            checked += 1
        s.rewind()
    assert checked == 5
    s.close()


@pytest.mark.parametrize("shape", [MODE5, MODE6])
def test_pair_rows_gulp_loop_candidates(hella, oracle, shape):
    params, sky = synth.config_plain(seed=15, nchan=160, gulp=2048, dm_max=300.0)
    sky.bursts[0].amp *= 4
    km = (np.random.default_rng(15).random(params["nchan"]) > 0.15).astype(np.int32)
    s = hella.Search(hella.default_params(**params))
    s.set_killmask(km)
    s.set_tuning(hella.HellaTuning(*shape))
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
    s.close()


def test_pair_rows_full_beam(hella):
    """The full single beam (2048 channels, 2501 trials): the whole plane
    identical to add mode 2's, both stage widths and both group sizes, and
    faster."""
    params, sky = synth.config_full(seed=2)
    s = _window(hella, params, sky)
    s.set_tuning(hella.HellaTuning(0, 4, 8, 0, 8, 2))
    s.dedisperse(0)
    ref = s.copy_dedisp()
    for shape in (MODE5, MODE5_16, MODE6):
        s.set_tuning(hella.HellaTuning(*shape))
        s.dedisperse(0)
        assert np.array_equal(s.copy_dedisp(), ref), shape
    ms6 = s.time_dedisp(hella.HellaTuning(*MODE6), 3)
    ms5 = s.time_dedisp(hella.HellaTuning(*MODE5_16), 3)
    ms2 = s.time_dedisp(hella.HellaTuning(0, 4, 8, 0, 8, 2), 3)
    print(f"full beam dedispersion (rows built and summed): add mode 6 {ms6:.2f} ms, add mode 5 {ms5:.2f} ms, "
          f"add mode 2 {ms2:.2f} ms")
    assert ms5 < ms2 and ms6 < ms2
    s.close()


def test_pair_rows_budget_and_batch(hella):
    """The rows count against the HBM budget: a budget with room for the
    context but not for the rows refuses the mode, and the tuner passes
    over it."""
    params, sky = synth.config_plain(seed=16, nchan=256, gulp=2048, dm_max=1000.0)
    held = hella.Search(hella.default_params(**params))
    dev = held.info.device_bytes
    held.close()
    s = hella.Search(hella.default_params(**params, hbm_budget=1 << 40))
    s.set_tuning(hella.HellaTuning(*MODE5))
    s.time_dedisp(None, 1)  # an ample budget
    s.close()
    # the smallest budget (to 64 KiB) the context is created with
    lo, hi = 0, dev + (64 << 20)
    while hi - lo > (64 << 10):
        mid = (lo + hi) // 2
        try:
            hella.Search(hella.default_params(**params, hbm_budget=mid)).close()
            hi = mid
        except hella.HellaError:
            lo = mid
    ntt = -(-(params["gulp"] + params["width_max"]) // 1024)
    rows_at_least = (params["nchan"] // 2) * ((ntt - 1) * 1024 + 512) * 4  # one row per pair
    assert hi - dev < rows_at_least, (hi, dev)
    s = hella.Search(hella.default_params(**params, hbm_budget=hi))
    s.set_tuning(hella.HellaTuning(*MODE5))
    with pytest.raises(hella.HellaError):
        s.time_dedisp(None, 1)
    best, _ = s.autotune(1)
    assert best.add_mode != 5
    s.close()


@pytest.mark.parametrize("shape", [MODE5, MODE5_16, MODE6])
def test_pair_rows_batch_killmasks(hella, shape):
    """The batched context in add mode 5 (the plan's rows over every channel,
    killed channels packed as zeros, each beam building the rows its own DM
    ceiling uses, beam by beam in one row buffer inside the gulp's graph)
    against single-beam contexts: candidates and planes identical."""
    params, _ = synth.config_plain(seed=44, nchan=128, gulp=2048, dm_max=400.0)
    nb = 5
    rng = np.random.default_rng(45)
    ceilings = np.array([400.0, 250.0, 330.0, 120.0, 400.0], np.float32)
    kill = (rng.random((nb, 128)) > rng.uniform(0, 0.1, (nb, 1))).astype(np.int32)
    kill[1] = 0
    kill[1, 77] = 1
    kill[3, :9] = 0
    skies = []
    for b in range(nb):
        sk = synth.config_plain(seed=46 + b, nchan=128, gulp=2048, dm_max=float(ceilings[b]))[1]
        sk.bursts[0].amp *= 3
        skies.append(sk)
    bt = hella.Batch(hella.default_params(**dict(params, nbeam=nb)), dm_max=ceilings, killmask=kill,
                     use_graph=True)
    bt.set_tuning(hella.HellaTuning(*shape))
    singles = []
    for b in range(nb):
        s = hella.Search(hella.default_params(**dict(params, dm_max=float(ceilings[b]), beam0=b, nbeam=1)))
        s.set_killmask(kill[b])
        singles.append(s)
    total = 0
    for g in range(max(s.info.min_gulp for s in singles) + 3):
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
    assert bt.get_tuning().add_mode == shape[5]
    bt.close()
    for s in singles:
        s.close()


def test_autotune_keeps_sums_exact(hella, oracle):
    """The tuner times every add mode including pair rows; whatever it keeps
    gives the oracle's plane."""
    params, sky = synth.config_plain(seed=17, nchan=256, gulp=4096, dm_max=1000.0)
    s = _window(hella, params, sky)
    win = s.copy_window(0)
    best, ms = s.autotune(1)
    assert s.get_tuning().add_mode == best.add_mode and ms > 0
    s.dedisperse(0)
    assert np.array_equal(s.copy_dedisp(), _oracle_plane(oracle, params, s, win, None))
    s.close()


def test_plan_api_pair_rows(hella, oracle):
    """hdd_set_pair_rows: hdd_execute_adv / hdd_execute_guru through pair rows
    give the channel-by-channel kernel's sums and the oracle's, with a
    killmask, host and device pointers, HDD_ASYNC, sub-ranges of trials and
    a sample count that changes between calls; switched off, the plan goes
    back to the channel-by-channel kernel."""
    torch = pytest.importorskip("torch")
    nch = 256
    plan = hella.Plan(nch, 1e-3, 468.75, -(468.75 - 375.0) / nch)
    plan.generate_dm_list(0.0, 1000.0, 40.0, 1.25)
    km = (np.random.default_rng(70).random(nch) > 0.07).astype(np.int32)
    plan.set_killmask(km)
    rng = np.random.default_rng(71)
    for extra, group in ((5000, 2), (2300, 2), (3100, 4)):
        x = rng.integers(0, 256, (plan.max_delay + extra, nch), dtype=np.uint8)
        plan.set_pair_rows(0)
        ref = plan.dedisperse(x)
        plan.set_pair_rows(group)
        got = plan.dedisperse(x)
        assert np.array_equal(got, ref), extra
        assert np.array_equal(got, oracle.dedisperse(x, plan.delay_table(), killmask=km, nout=extra)), extra
    with pytest.raises(hella.HellaError):
        plan.set_pair_rows(3)
    # a sub-range of trials, device pointers, asynchronous
    nsamps, nout = x.shape[0], x.shape[0] - plan.max_delay
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    dx = torch.from_numpy(x).cuda()
    first, count = 37, 100
    out = torch.full((count, nout), -1.0, dtype=torch.float32, device="cuda")
    plan.execute_guru(nsamps, dx, nch, out, nout * 4, first, count,
                      flags=hella.HDD_DEVICE_POINTERS | hella.HDD_ASYNC)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref[first:first + count])
    plan.set_pair_rows(0)
    assert np.array_equal(plan.dedisperse(x), ref)
    plan.close()


@pytest.mark.parametrize("shape", [MODE5, MODE6])
def test_pair_rows_batch_chunks(hella, shape):
    """19 beams: rows built and summed 4 beams per launch pair (4 x 4 + 3),
    DM ceilings from 60 to 300 and killmasks differing per beam; every
    beam's plane and candidates identical to its single-beam context."""
    nb, nch = 19, 64
    params, _ = synth.config_plain(seed=95, nchan=nch, gulp=1024, dm_max=300.0)
    rng = np.random.default_rng(96)
    ceilings = rng.uniform(60.0, 300.0, nb).astype(np.float32)
    ceilings[[0, 9]] = 300.0
    kill = (rng.random((nb, nch)) > rng.uniform(0, 0.15, (nb, 1))).astype(np.int32)
    skies = []
    for b in range(nb):
        sk = synth.config_plain(seed=97 + b, nchan=nch, gulp=1024, dm_max=float(ceilings[b]))[1]
        sk.bursts[0].amp *= 4
        skies.append(sk)
    bt = hella.Batch(hella.default_params(**dict(params, nbeam=nb)), dm_max=ceilings, killmask=kill)
    bt.set_tuning(hella.HellaTuning(*shape))
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
    bt.close()
    for s in singles:
        s.close()
