"""GPU parity: every stage of the GB300 path through the C ABI against the
oracle on the same seeded inputs.  Integer and byte results (ring bytes,
dedispersed sums, candidate indices) must be bit-exact; normalised fp32
planes are checked bit-exact too, and against the 1e-5 relative tolerance
the search contract states."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline, small_params

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # normalised fp32 outputs


def _search(hella, params, **over):
    p = dict(params)
    p.update(over)
    return hella.Search(hella.default_params(**p))


# ----------------------------------------------------------------- fp16

def test_fp16_intrinsics_correctly_rounded(hella):
    bad, first = hella.fp16_selftest(0)
    assert bad == 0, hex(first)


# ------------------------------------------------------------ dedisp API

def _random_plan(hella, nchan=256, dm_max=150.0, dt=1e-3):
    plan = hella.Plan(nchan, dt, 468.75, -(468.75 - 375.0) / nchan)
    plan.generate_dm_list(0.0, dm_max, 40.0, 1.25)
    return plan


def test_dedisp_exact_random(hella, oracle):
    plan = _random_plan(hella)
    rng = np.random.default_rng(10)
    nsamps = plan.max_delay + 3000
    x = rng.integers(0, 256, (nsamps, plan.nchans), dtype=np.uint8)
    got = plan.dedisperse(x)
    want = oracle.dedisperse(x, plan.delay_table())
    assert np.array_equal(got, want)


def test_dedisp_killmask_stride_guru(hella, oracle):
    plan = _random_plan(hella, nchan=320, dm_max=200.0)
    rng = np.random.default_rng(11)
    km = (rng.random(plan.nchans) > 0.1).astype(np.int32)
    plan.set_killmask(km)
    nsamps, stride = plan.max_delay + 2500, plan.nchans + 48
    x = rng.integers(0, 256, (nsamps, stride), dtype=np.uint8)
    nout = nsamps - plan.max_delay
    first, count = 17, plan.dm_count - 30
    ostride = nout + 5
    out = np.full((count, ostride), -1.0, np.float32)
    plan.execute_guru(nsamps, x, stride, out, ostride * 4, first, count)
    want = oracle.dedisperse(np.ascontiguousarray(x[:, :plan.nchans]), plan.delay_table()[first:first + count],
                             killmask=km, nout=nout)
    assert np.array_equal(out[:, :nout], want)
    assert np.all(out[:, nout:] == -1.0)  # padding untouched


def test_dedisp_device_pointers(hella, oracle):
    torch = pytest.importorskip("torch")
    plan = _random_plan(hella, nchan=128, dm_max=80.0)
    rng = np.random.default_rng(12)
    nsamps = plan.max_delay + 1500
    x = rng.integers(0, 256, (nsamps, plan.nchans), dtype=np.uint8)
    nout = nsamps - plan.max_delay
    dx = torch.from_numpy(x).cuda()
    dout = torch.empty((plan.dm_count, nout), dtype=torch.float32, device="cuda")
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    plan.execute_adv(nsamps, dx, plan.nchans, dout, nout * 4, flags=hella.HDD_DEVICE_POINTERS)
    assert np.array_equal(dout.cpu().numpy(), oracle.dedisperse(x, plan.delay_table()))


def test_dedisp_sparse_dm_list_uses_small_tiles(hella, oracle):
    """Widely spaced trials make every tile's delay spread large; the kernel
    falls back to smaller DM tiles and must stay exact."""
    plan = hella.Plan(512, 1e-3, 468.75, -0.18)
    plan.set_dm_list(np.linspace(0, 1500, 40, dtype=np.float32))
    rng = np.random.default_rng(13)
    nsamps = plan.max_delay + 1200
    x = rng.integers(0, 256, (nsamps, plan.nchans), dtype=np.uint8)
    assert np.array_equal(plan.dedisperse(x), oracle.dedisperse(x, plan.delay_table()))


def test_dedisp_unsorted_dm_list(hella, oracle):
    """A DM list in no particular order (descending runs, repeats, a jump
    back to 0): tiles span each channel's smallest to largest delay, and
    the output length follows the largest delay of any trial."""
    plan = hella.Plan(256, 1e-3, 468.75, -(468.75 - 375.0) / 256)
    rng = np.random.default_rng(14)
    dms = np.concatenate([np.linspace(300, 0, 37), [0.0, 0.0, 250.0], rng.uniform(0, 400, 29),
                          np.linspace(10, 60, 20)]).astype(np.float32)
    plan.set_dm_list(dms)
    assert plan.max_delay == plan.delay_table().max() > plan.delay_table()[-1].max()
    nsamps = plan.max_delay + 2100
    x = rng.integers(0, 256, (nsamps, plan.nchans), dtype=np.uint8)
    assert np.array_equal(plan.dedisperse(x), oracle.dedisperse(x, plan.delay_table()))


def test_dedisp_constant_input(hella):
    plan = _random_plan(hella, nchan=384, dm_max=120.0)
    x = np.full((plan.max_delay + 777, plan.nchans), 128, np.uint8)
    assert np.all(plan.dedisperse(x) == 128 * plan.nchans)


# -------------------------------------------------------- search stages

def _run_to_search(hella, oracle, params, sky, beams=1):
    """Feed gulps until the first searched one; returns (search, oracle
    pipeline, last gulp)."""
    s = _search(hella, params, nbeam=beams)
    pl = oracle_pipeline(oracle, params, nbeam=beams)
    assert s.info.ntime == pl.ntime and s.info.ndms == pl.ndms and s.info.min_gulp == pl.min_gulp
    G = params["gulp"]
    for g in range(pl.min_gulp):
        x = np.stack([sky.gulp(g, G)] * beams) if beams > 1 else sky.gulp(g, G)[None]
        c, searched = s.process_gulp(x)
        c2, searched2 = pl.gulp_step(x)
        assert not searched and not searched2
    return s, pl


@pytest.mark.parametrize("nchan", [256, 96, 160])  # 96, 160: partial 128-channel slices
def test_flagger_bit_exact(hella, oracle, nchan):
    p = small_params(nchan=nchan, gulp=4096)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=21, rfi_chans=(3, 50), slope=0.4)
    s = _search(hella, p)
    x = sky.gulp(0, p["gulp"])
    x[:, 77] = 0  # a dead channel (spectral flag)
    s.load_gulp(x[None])
    s.fast_flagger()
    win = s.copy_window(0)
    out, ts, tr = oracle.flag_beam(x)
    st = s.flag_stats(0)
    for k in ("bp1", "bp2", "bp3"):
        assert np.array_equal(st[k].view(np.uint32), tr[k].view(np.uint32)), k
    for k in ("mean1", "std1", "mean2", "std2"):
        assert np.float32(st[k]).view(np.uint32) == np.float32(tr[k]).view(np.uint32), k
    assert np.array_equal(st["ts"].view(np.uint32), ts.view(np.uint32))
    assert np.array_equal(win[-p["gulp"]:], out)


def test_search_stages_bit_exact(hella, oracle):
    params, sky = synth.config_plain(seed=5, nchan=256, gulp=4096, dm_max=400.0)
    s, pl = _run_to_search(hella, oracle, params, sky)
    g = pl.min_gulp
    x = sky.gulp(g, params["gulp"])[None]
    s.clear_peaks()
    s.load_gulp(x)
    s.fast_flagger()
    win = s.copy_window(0)
    c_or, _ = pl.gulp_step(x)  # oracle: flag + search + rewind
    ref = pl.search_window(win, 0)
    s.dedisperse(0)
    assert np.array_equal(s.copy_dedisp(), ref["dd"])
    s.smooth(1)
    mean, std, s0 = s.smooth_stats()
    assert np.array_equal(mean.view(np.uint32), ref["mean"].view(np.uint32))
    assert np.array_equal(std.view(np.uint32), ref["std"].view(np.uint32))
    boxes = s.copy_boxes()
    assert np.allclose(boxes, ref["boxes"], rtol=RTOL, atol=RTOL)
    assert np.array_equal(boxes.view(np.uint32), ref["boxes"].view(np.uint32))
    s.find_peaks(0)
    got = s.get_peaks()
    assert np.float32(s0).view(np.uint32) == np.float32(ref["sigma0"]).view(np.uint32)
    assert cands_equal(got, ref["cands"])
    assert cands_equal(got, c_or)
    assert len(got) > 0


@pytest.mark.parametrize("wmin,wmax,anchor", [
    (1, 16, 1),     # span 16: k_firR, stride 133
    (3, 400, 1),    # odd widths 3..384, span 768: stride 257, odd window offsets
    (1, 2048, 0),   # widths up to 1024, span 2048: the largest k_firR stride
    (1, 4096, 1),   # span 4096: the k_fir fallback
    (5, 11, 0),     # a single width
])
def test_smoothing_width_sets_bit_exact(hella, oracle, wmin, wmax, anchor):
    """Smoothed planes, per-width statistics and candidates for width sets
    that take each FIR kernel and shared-memory stride."""
    p = small_params(nchan=128, gulp=4096, dm_max=60.0, width_min=wmin, width_max=wmax, smooth_anchor=anchor,
                     snr=5.0)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=31 + wmin, rfi_chans=(9,), slope=0.2)
    s, pl = _run_to_search(hella, oracle, p, sky)
    x = sky.gulp(pl.min_gulp, p["gulp"])[None]
    s.clear_peaks()
    s.load_gulp(x)
    s.fast_flagger()
    win = s.copy_window(0)
    pl.gulp_step(x)
    ref = pl.search_window(win, 0)
    s.dedisperse(0)
    s.smooth(1)
    mean, std, s0 = s.smooth_stats()
    boxes = s.copy_boxes()
    assert boxes.shape == ref["boxes"].shape
    assert np.array_equal(boxes.view(np.uint32), ref["boxes"].view(np.uint32))
    assert np.array_equal(mean.view(np.uint32), ref["mean"].view(np.uint32))
    assert np.array_equal(std.view(np.uint32), ref["std"].view(np.uint32))
    s.find_peaks(0)
    assert cands_equal(s.get_peaks(), ref["cands"])


@pytest.mark.parametrize("nchan", [96, 160])
def test_gulp_loop_partial_channel_slices(hella, oracle, nchan):
    """Channel counts that are not multiples of the flagger's 128-channel
    slices: candidates of a whole gulp loop identical to the oracle's."""
    params, sky = synth.config_plain(seed=11, nchan=nchan, gulp=2048, dm_max=300.0)
    sky.bursts[0].amp *= 4
    s = _search(hella, params)
    pl = oracle_pipeline(oracle, params)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, params["gulp"])[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so
        assert cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0


def test_gulp_loop_killmask(hella, oracle):
    """A dedisp killmask (a fifth of the channels, runs of them and single
    ones): candidates of a whole gulp loop identical to the oracle's."""
    params, sky = synth.config_plain(seed=14, nchan=160, gulp=2048, dm_max=300.0)
    sky.bursts[0].amp *= 4
    rng = np.random.default_rng(14)
    km = (rng.random(params["nchan"]) > 0.15).astype(np.int32)
    km[40:56] = 0
    s = _search(hella, params)
    s.set_killmask(km)
    pl = oracle_pipeline(oracle, params)
    pl.set_killmask(0, km)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, params["gulp"])[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so
        assert cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0


@pytest.mark.parametrize("gulp", [256, 1056, 2080])
def test_gulp_loop_ragged_gulps(hella, oracle, gulp):
    """Gulps that are not multiples of the FIR's 2048-sample chunks, the ring
    writer's 512-sample tiles or the statistics' 256 columns: candidates and
    the smoothed planes of the last gulp identical to the oracle's."""
    params, sky = synth.config_plain(seed=12, nchan=128, gulp=gulp, dm_max=150.0)
    params["snr"] = 4.0
    s = _search(hella, params)
    pl = oracle_pipeline(oracle, params)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, gulp)[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so
        assert cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0


@pytest.mark.parametrize("anchor", [0, 1])
def test_gulp_loop_multibeam(hella, oracle, anchor):
    params, _ = synth.config_plain(seed=7, nchan=128, gulp=2048, dm_max=400.0)
    params["smooth_anchor"] = anchor
    skies = [synth.config_plain(seed=70 + b, nchan=128, gulp=2048, dm_max=400.0)[1] for b in range(3)]
    for sk in skies:
        sk.bursts[0].amp *= 3
    s = _search(hella, params, nbeam=3, beam0=0)
    pl = oracle_pipeline(oracle, params, nbeam=3)
    total = 0
    for g in range(pl.min_gulp + 3):
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so
        assert cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0


def test_max_giants_cap(hella, oracle):
    params, sky = synth.config_plain(seed=9, nchan=128, gulp=2048, dm_max=400.0)
    sky.bursts[0].amp *= 6
    params.update(max_giants=25, snr=3.0)
    s = _search(hella, params, nbeam=2)
    pl = oracle_pipeline(oracle, params, nbeam=2)
    for g in range(pl.min_gulp + 1):
        x = np.stack([sky.gulp(g, params["gulp"])] * 2)
        got, _ = s.process_gulp(x)
        want, _ = pl.gulp_step(x)
        assert cands_equal(got, want)
    assert len(got) == 25


def test_plain_config_full_size(hella, oracle):
    """512 channels, gulp 16384, DM 0-500: candidates bit-exact and the
    injected DM-300 burst recovered within 2 pc/cm^3 (verify_injection_fil.py:30-40)."""
    params, sky = synth.config_plain(seed=1)
    s = _search(hella, params)
    pl = oracle_pipeline(oracle, params)
    for g in range(pl.min_gulp + 1):
        x = sky.gulp(g, params["gulp"])[None]
        got, searched = s.process_gulp(x)
        want, _ = pl.gulp_step(x)
        assert cands_equal(got, want)
    assert searched and len(got)
    best = got[np.argmax(got["snr"])]
    assert abs(s.dm_list()[best["dm_idx"]] - 300.0) < 2.0


def test_always_find_peaks_switch(hella, oracle):
    """DEBUG_ALWAYS_FIND_PEAKS (definitions.h:66) as `always_find_peaks`: a
    gulp loop with the gate off gives the oracle's candidates with its gate
    off (here sigma0 is near 1, so also the gated ones)."""
    params, sky = synth.config_plain(seed=19, nchan=128, gulp=2048, dm_max=200.0)
    params["always_find_peaks"] = 1
    sky.bursts[0].amp *= 3
    s = _search(hella, params)
    pl = oracle_pipeline(oracle, params)
    total = 0
    for g in range(pl.min_gulp + 2):
        x = sky.gulp(g, params["gulp"])[None]
        got, sg = s.process_gulp(x)
        want, so = pl.gulp_step(x)
        assert sg == so and cands_equal(got, want), (g, len(got), len(want))
        total += len(got)
    assert total > 0
