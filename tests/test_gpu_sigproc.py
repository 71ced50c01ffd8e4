"""The SIGPROC input loop: a filterbank file whose header was written by the
reference's own header writer (tests/golden/ref_header.fil: 64 channels,
fch1 468.75 MHz, tsamp 1.048576 ms) followed by synthetic u8 spectra is read
gulp by gulp through hella_fil_read and searched with the parameters the
header gives; candidates equal the oracle's on the same spectra."""
from pathlib import Path

import numpy as np
import pytest

import synth
from helpers import cands_equal, oracle_pipeline, small_params

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def test_filterbank_file_feeds_the_search(hella, oracle, tmp_path):
    ref = GOLD / "ref_header.fil"
    h = hella.Filterbank(ref, 64).header
    head = ref.read_bytes()[: h.header_bytes]
    G = 2048
    p = small_params(nchan=h.nchans, gulp=G, tsamp=h.tsamp, plan_dt=h.tsamp, f0_mhz=h.fch1, df_mhz=h.foff,
                     dm_max=200.0, snr=4.0)
    sky = synth.Sky(h.nchans, h.tsamp, h.fch1, h.foff, seed=47, rfi_chans=(7,), slope=0.2)
    pl = oracle_pipeline(oracle, p)
    ngulp = pl.min_gulp + 3
    data = np.concatenate([sky.gulp(g, G) for g in range(ngulp)])
    path = tmp_path / "search.fil"
    path.write_bytes(head + data.tobytes())

    f = hella.Filterbank(path, 64)
    s = hella.Search(hella.default_params(**p))
    total, g = 0, 0
    while True:
        x = f.read(G)
        if len(x) < G:
            assert len(x) == 0
            break
        got, searched = s.process_gulp(x[None])
        want, so = pl.gulp_step(sky.gulp(g, G)[None])
        assert searched == so and cands_equal(got, want), g
        total += len(got)
        g += 1
    assert g == ngulp and total > 0
