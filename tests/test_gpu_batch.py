"""Batched multi-beam search: every beam's candidates and dedispersed plane
must equal, bit for bit, those of a single-beam context created with that
beam's DM ceiling and killmask and fed the same gulps (the contract of the
batched configuration: output equal to independent plain runs)."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline

pytestmark = pytest.mark.gpu

NB = 6


def _setup(seed=40, nchan=128, gulp=2048):
    params, _ = synth.config_plain(seed=seed, nchan=nchan, gulp=gulp, dm_max=400.0)
    rng = np.random.default_rng(seed)
    ceilings = np.array([400.0, 250.0, 330.0, 180.0, 400.0, 300.0], np.float32)[:NB]
    kill = (rng.random((NB, nchan)) > rng.uniform(0, 0.1, (NB, 1))).astype(np.int32)
    skies = []
    for b in range(NB):
        sk = synth.config_plain(seed=seed + 1 + b, nchan=nchan, gulp=gulp, dm_max=float(ceilings[b]))[1]
        sk.bursts[0].amp *= 3
        skies.append(sk)
    return params, ceilings, kill, skies


def _single(hella, params, ceiling, kill, beam):
    p = dict(params, dm_max=float(ceiling), beam0=beam, nbeam=1)
    s = hella.Search(hella.default_params(**p))
    s.set_killmask(kill)
    return s


@pytest.mark.parametrize("use_graph,wpp", [(True, 0), (False, 2)])
def test_batch_equals_independent_runs(hella, use_graph, wpp):
    params, ceilings, kill, skies = _setup()
    _compare(hella, params, ceilings, kill, skies, widths_per_pass=wpp, use_graph=use_graph)


def test_batch_with_median_window_and_gate_off(hella, oracle):
    """The runtime NMEDFILT and DEBUG_ALWAYS_FIND_PEAKS reach every beam of
    the batch: equal to single-beam contexts and oracle pipelines with them."""
    params, ceilings, kill, skies = _setup(seed=47)
    params.update(bp_median=5, always_find_peaks=1)
    _compare(hella, params, ceilings, kill, skies, oracle=oracle)


def test_batch_killmask_extremes(hella, oracle):
    """Beams that kill every channel, all but one, none, every other one,
    and the first 8 (a whole staging step): each beam sums only its own
    channels and equals its single-beam context and an oracle pipeline with
    its DM ceiling and killmask."""
    params, ceilings, kill, skies = _setup(seed=45)
    nchan = kill.shape[1]
    kill[0] = 0
    kill[1] = 0
    kill[1, 77] = 1
    kill[2] = 1
    kill[3] = np.arange(nchan) % 2
    kill[4, :8] = 0
    _compare(hella, params, ceilings, kill, skies, oracle=oracle)


def _compare(hella, params, ceilings, kill, skies, oracle=None, **batch_kw):
    base = hella.default_params(**dict(params, nbeam=NB))
    bt = hella.Batch(base, dm_max=ceilings, killmask=kill, **batch_kw)
    singles = [_single(hella, params, ceilings[b], kill[b], b) for b in range(NB)]
    pls = []
    if oracle is not None:
        for b in range(NB):
            pl = oracle_pipeline(oracle, params, dm_max=float(ceilings[b]))
            pl.set_killmask(0, kill[b])
            pls.append(pl)
    assert [bt.info(b).ndms for b in range(NB)] == [s.info.ndms for s in singles]
    assert [bt.info(b).ntime for b in range(NB)] == [s.info.ntime for s in singles]
    total = 0
    ngulp = max(s.info.min_gulp for s in singles) + 3
    for g in range(ngulp):
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        got, counts, searched = bt.process_gulp(x)
        off = 0
        for b, s in enumerate(singles):
            want, sw = s.process_gulp(x[b:b + 1])
            assert searched[b] == sw, (g, b)
            mine = got[off:off + counts[b]]
            off += counts[b]
            assert cands_equal(mine, want), (g, b, len(mine), len(want))
            if pls:
                ref, so = pls[b].gulp_step(x[b:b + 1])
                ref["beam"] = b
                assert so == sw and cands_equal(mine, ref), (g, b, len(mine), len(ref))
            if sw:
                assert np.array_equal(bt.copy_dedisp(b), s.copy_dedisp()), (g, b)
            total += len(want)
        assert off == len(got)
    assert total > 0


def test_batch_tile_shapes_agree(hella):
    params, ceilings, kill, skies = _setup(seed=50)
    base = hella.default_params(**dict(params, nbeam=NB))
    outs = []
    for t in [(0, 4, 8, 0, 8, 0), (8, 4, 16, 2, 1, 1), (16, 4, 8, 3, 4, 2), (16, 4, 16, 2, 8, 3)]:
        bt = hella.Batch(base, dm_max=ceilings, killmask=kill)
        bt.set_tuning(hella.HellaTuning(*t))
        res = []
        for g in range(bt.info(0).min_gulp + 2):
            got, counts, _ = bt.process_gulp(synth.multibeam_gulp(skies, g, params["gulp"]))
            res.append((got.copy(), counts.copy()))
        outs.append((res, [bt.copy_dedisp(b) for b in range(NB)]))
        bt.close()
    for res, dd in outs[1:]:
        for (a, ca), (b, cb) in zip(outs[0][0], res):
            assert np.array_equal(ca, cb) and cands_equal(a, b)
        for a, b in zip(outs[0][1], dd):
            assert np.array_equal(a, b)


def test_batch_autotune_keeps_results(hella):
    params, ceilings, kill, skies = _setup(seed=60)
    base = hella.default_params(**dict(params, nbeam=NB))
    bt = hella.Batch(base, dm_max=ceilings, killmask=kill)
    best, ms = bt.autotune(1)
    assert ms > 0 and hella.HellaTuning(**{k: getattr(best, k) for k, _ in best._fields_}).chan_chunk in (8, 16)
    ref = hella.Batch(base, dm_max=ceilings, killmask=kill)
    for g in range(bt.info(0).min_gulp + 2):
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        a, ca, _ = bt.process_gulp(x)
        b, cb, _ = ref.process_gulp(x)
        assert np.array_equal(ca, cb) and cands_equal(a, b)
