"""The DADA input path (INPUT DADA: fp16 gulps in channel-major order,
casm_hella_refactored.cu:78,245-248,688-691; transpose.cu:87-90): flagger
output and candidates bit-exact against the oracle fed the same fp16 gulps,
for the single-beam context (with and without SCRUNCH entries) and the batch."""
import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline, small_params

pytestmark = pytest.mark.gpu


def _f16_ft(x_u8: np.ndarray, seed: int) -> np.ndarray:
    """u8 [..., w, nchan] -> fp16 [..., nchan, w] with sub-integer detail, as a
    voltage beamformer's fp16 output would carry."""
    rng = np.random.default_rng(seed)
    f = x_u8.astype(np.float32) + rng.uniform(-0.45, 0.45, x_u8.shape).astype(np.float32)
    return np.ascontiguousarray(np.swapaxes(f.astype(np.float16), -1, -2))


@pytest.mark.parametrize("entries", [(), ((4, 2, 3.0, 1),)])
def test_dada_flagger_bit_exact(hella, oracle, entries):
    p = small_params(nchan=128, gulp=4096)
    sky = synth.Sky(p["nchan"], p["tsamp"], p["f0_mhz"], p["df_mhz"], seed=41, rfi_chans=(5, 90), slope=0.3)
    s = hella.Search(hella.default_params(**p, scrunches=list(entries), input_format=1))
    fspec = np.zeros(p["nchan"], np.float32)
    fp = oracle.flag_params(scrunches=list(entries))
    for g in range(2):
        x = sky.gulp(g, p["gulp"])
        x[:, 77] = 0
        ft = _f16_ft(x, g)
        s.load_gulp(ft[None])
        s.fast_flagger()
        out, ts, tr = oracle.flag_beam_f16(ft, fp, fspec)
        st = s.flag_stats(0)
        for k in ("bp1", "bp2", "bp3"):
            assert np.array_equal(st[k].view(np.uint32), tr[k].view(np.uint32)), (g, k)
        for k in ("mean1", "std1", "mean2", "std2"):
            assert np.float32(st[k]).view(np.uint32) == np.float32(tr[k]).view(np.uint32), (g, k)
        assert np.array_equal(st["ts"].view(np.uint32), ts.view(np.uint32))
        assert np.array_equal(s.copy_window(0)[-p["gulp"]:], out), g
        s.rewind()


@pytest.mark.parametrize("add_mode", [None, 6])
def test_dada_gulp_loop_and_batch(hella, oracle, add_mode):
    """add_mode 6: both contexts dedisperse through quad rows."""
    params, _ = synth.config_plain(seed=43, nchan=128, gulp=2048, dm_max=400.0)
    skies = [synth.config_plain(seed=44 + b, nchan=128, gulp=2048, dm_max=400.0)[1] for b in range(2)]
    for sk in skies:
        sk.bursts[0].amp *= 3
    s = hella.Search(hella.default_params(**dict(params, nbeam=2), input_format=1))
    bt = hella.Batch(hella.default_params(**dict(params, nbeam=2), input_format=1))
    if add_mode:
        s.set_tuning(hella.HellaTuning(16, 4, 16, 0, 4, add_mode))
        bt.set_tuning(hella.HellaTuning(16, 4, 16, 0, 4, add_mode))
    pl = oracle_pipeline(oracle, params, nbeam=2)
    total = 0
    for g in range(pl.min_gulp + 2):
        ft = _f16_ft(synth.multibeam_gulp(skies, g, params["gulp"]), 100 + g)
        got, _ = s.process_gulp(ft)
        want, _ = pl.gulp_step_f16(ft)
        assert cands_equal(got, want), g
        bgot, _, _ = bt.process_gulp(ft)
        assert cands_equal(bgot, want), g
        total += len(got)
    assert total > 0


def test_dada_ring_feeds_the_search(hella, oracle):
    """The DADA loop (casm_hella_refactored.cu:662-670,688-691): a writer
    thread puts the header and fp16 channel-major gulps into a pinned
    header/data ring; the reader takes TSAMP and UTC_START from the header,
    searches every block in place (hella_process_gulp on the ring's own
    pinned memory) and builds the coincidencer message; candidates equal the
    oracle's on the same gulps."""
    import threading

    params, sky = synth.config_plain(seed=45, nchan=128, gulp=2048, dm_max=400.0)
    sky.bursts[0].amp *= 3
    G, nch = params["gulp"], params["nchan"]
    pl = oracle_pipeline(oracle, params)
    ngulp = pl.min_gulp + 3
    blocks = [_f16_ft(sky.gulp(g, G), 200 + g) for g in range(ngulp)]
    ring = hella.Ring(G * nch * 2, 3, pinned=True)
    header = (f"HDR_VERSION 1.0\nUTC_START 2025-06-01-12:00:00\nPICOSECONDS 0\n"
              f"TSAMP {params['tsamp'] * 1e6:.3f}\nNCHAN {nch}\nNBIT 16\n")

    def produce():
        ring.write_header(header)
        for b in blocks:
            ring.write(b.tobytes(), timeout_ms=10000)
        ring.end()

    th = threading.Thread(target=produce)
    th.start()
    hdr = ring.read_header(10000)
    assert hella.header_get(hdr, "NCHAN") == str(nch)
    s = hella.Search(hella.default_params(**params, input_format=1))
    dms = s.dm_list()
    total, g = 0, 0
    while True:
        addr, n = ring.open_read(timeout_ms=10000)
        if n == 0:
            break
        assert n == G * nch * 2
        got, searched = s.process_gulp(addr)
        ring.mark_cleared()
        want, so = pl.gulp_step_f16(blocks[g][None])
        assert searched == so and cands_equal(got, want), g
        msg = hella.cands_coincidencer(g + 1, got, g * G, dms, utc_start=hella.header_get(hdr, "UTC_START"),
                                       picoseconds=hella.header_get(hdr, "PICOSECONDS"),
                                       tsamp=hella.header_get(hdr, "TSAMP"))
        assert msg.splitlines()[0] == f"{g + 1} 2025-06-01-12:00:00 0 {params['tsamp'] * 1e6:.3f}"
        assert len(msg.splitlines()) == 1 + len(got)
        total += len(got)
        g += 1
    th.join(timeout=30)
    ring.close()
    assert g == ngulp and total > 0
