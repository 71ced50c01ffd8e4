"""The full single-beam workload (2048 channels, gulp 65536, DM 0-2000 at
tolerance 1.25, 2501 trials) at full size: the flagger's output bytes of a
whole gulp and 48 sampled dedispersed trials of the first searched window
bit-exact against the oracle, and the candidate lists of two contexts fed the
same gulps identical (determinism)."""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


def test_full_beam_flagger_and_dedisp_rows(hella, oracle):
    params, sky = synth.config_full(seed=2)
    G = params["gulp"]
    s = hella.Search(hella.default_params(**params))
    info = s.info
    oracle.set_threads(0)
    for g in range(info.min_gulp + 1):
        x = sky.gulp(g, G)
        s.clear_peaks()
        s.load_gulp(x[None])
        s.fast_flagger()
        if g == 0:
            out, _, _ = oracle.flag_beam(x)
            assert np.array_equal(s.copy_window(0)[-G:], out)
        if g < info.min_gulp:
            s.rewind()
    win = s.copy_window(0)
    s.dedisperse(0)
    dd = s.copy_dedisp()
    dms = s.dm_list()
    f32 = lambda v: float(np.float32(v))
    delays = oracle.dm_delays(dms, oracle.delay_table(params["nchan"], f32(params["plan_dt"]),
                                                      f32(params["f0_mhz"]), f32(params["df_mhz"])))
    rows = np.unique(np.linspace(0, len(dms) - 1, 48).astype(int))
    want = oracle.dedisperse(win, delays[rows], nout=info.ntime_dd)
    assert np.array_equal(dd[rows], want)


def test_full_beam_deterministic(hella):
    params, sky = synth.config_full(seed=2)
    G = params["gulp"]
    a = hella.Search(hella.default_params(**params))
    b = hella.Search(hella.default_params(**params, autotune=1))
    counts = []
    for g in range(a.info.min_gulp + 3):
        x = sky.gulp(g, G)[None]
        ca, sa = a.process_gulp(x)
        cb, sb = b.process_gulp(x)
        assert sa == sb and len(ca) == len(cb)
        assert np.array_equal(ca, cb)
        counts.append(len(ca))
    assert counts[-1] > 0
