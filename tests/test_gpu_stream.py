"""Streaming serving loop: slots join and leave a dynamic batch between
gulps while two gulps are in flight; every slot's candidates must equal
those of a single-beam context started when the slot joined, fed the same
gulps, and its running bandpass must be the exponentially weighted mean of
that context's calc_bandpass_new output."""
import numpy as np
import pytest

import synth
from helpers import cands_equal

pytestmark = pytest.mark.gpu

NS = 5          # slots
ALPHA = 0.25


def _ew(prev, bp):
    """fp32 ew + alpha * (bp - ew), each operation rounded."""
    a = np.float32(ALPHA)
    return (prev + (a * (bp - prev).astype(np.float32)).astype(np.float32)).astype(np.float32)


@pytest.mark.parametrize("add_mode", [None, 6])
def test_stream_join_leave_matches_fresh_contexts(hella, add_mode):
    """add_mode 6: the dedispersion through quad rows, built and summed for
    several slots per launch pair, slots without trials among them."""
    params, _ = synth.config_plain(seed=80, nchan=128, gulp=2048, dm_max=400.0)
    rng = np.random.default_rng(80)
    skies = []
    for b in range(NS):
        sk = synth.config_plain(seed=81 + b, nchan=128, gulp=2048, dm_max=400.0)[1]
        sk.bursts[0].amp *= 3
        skies.append(sk)
    base = hella.default_params(**dict(params, nbeam=NS))
    member = [1, 1, 1, 0, 0]
    bt = hella.Batch(base, dynamic=True, member=member, inflight=2, bp_alpha=ALPHA)
    if add_mode:
        bt.set_tuning(hella.HellaTuning(16, 4, 16, 0, 4, add_mode))
    # membership events before gulp g: (slot, member, dm_max, killmask)
    km3 = (rng.random(128) > 0.08).astype(np.int32)
    events = {3: [(3, 1, 250.0, km3)], 5: [(1, 0, 0.0, None)], 6: [(4, 1, 400.0, None)]}
    ctx = {b: (hella.Search(hella.default_params(**dict(params, nbeam=1, beam0=b))), None) for b in range(3)}
    ew = {b: None for b in range(NS)}
    ngulp = 12
    pending = []   # (gulp index, {slot: expected cands}, {slot: searched})

    def expect(g, x):
        want, sw = {}, {}
        for b, (s, _) in ctx.items():
            c, searched = s.process_gulp(x[b:b + 1])
            want[b], sw[b] = c, searched
            bp1 = s.flag_stats(0)["bp1"]
            ew[b] = bp1.copy() if ew[b] is None else _ew(ew[b], bp1)
        return want, sw

    def check(item, res):
        g, want, sw = item
        got, counts, searched, lat, dev = res
        assert lat >= dev * 0.5 and dev > 0
        off = 0
        for b in range(NS):
            mine = got[off:off + counts[b]]
            off += counts[b]
            if b in want:
                assert searched[b] == sw[b], (g, b)
                assert cands_equal(mine, want[b]), (g, b, len(mine), len(want[b]))
            else:
                assert counts[b] == 0 and not searched[b]

    found = 0
    for g in range(ngulp):
        if g in events:
            while pending:                      # membership changes need an idle batch
                item = pending.pop(0)
                check(item, bt.poll())
            for slot, m, dmx, km in events[g]:
                bt.set_beam(slot, m, dmx, km)
                if m:
                    s = hella.Search(hella.default_params(**dict(params, nbeam=1, beam0=slot, dm_max=dmx)))
                    if km is not None:
                        s.set_killmask(km)
                    ctx[slot] = (s, g)
                    ew[slot] = None
                else:
                    ctx.pop(slot)
        x = synth.multibeam_gulp(skies, g, params["gulp"])
        bt.submit(x)
        want, sw = expect(g, x)
        found += sum(len(v) for v in want.values())
        pending.append((g, want, sw))
        if len(pending) == 2:
            item = pending.pop(0)
            check(item, bt.poll())
    while pending:
        item = pending.pop(0)
        check(item, bt.poll())
    assert found > 0
    for b in ctx:
        assert np.array_equal(bt.bandpass(b), ew[b]), b


def test_admission_by_budget(hella):
    """hella_batch_bytes sizes a batch; creation within the budget succeeds,
    one slot more than fits is refused (all 6 widths held per pass)."""
    params, _ = synth.config_plain(seed=90, nchan=128, gulp=2048, dm_max=400.0)
    kw = dict(dynamic=True, inflight=2, widths_per_pass=6)
    size = {n: hella.batch_bytes(hella.default_params(**dict(params, nbeam=n)), **kw) for n in (1, 4, 5)}
    assert size[4] > 3 * size[1]
    budget = (size[4] + size[5]) // 2
    ok = hella.Batch(hella.default_params(**dict(params, nbeam=4, hbm_budget=budget)), **kw)
    ok.close()
    with pytest.raises(hella.HellaError, match="budget"):
        hella.Batch(hella.default_params(**dict(params, nbeam=5, hbm_budget=budget)), **kw)
