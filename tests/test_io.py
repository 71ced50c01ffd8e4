"""The host-side data paths around the search (include/hella_io.h): the
SIGPROC reader against a file written by the reference's own header writer
(tests/golden/ref_header.fil), the candidate line formats of output_peaks,
clustering, flag statistics, the in-process ring and DADA header parsing
against a header from the reference's converter (tests/golden/ref_dada_header.txt)."""
import struct
import threading

import numpy as np
import pytest

GOLD = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _w(fh, s):
    b = s.encode()
    fh.write(struct.pack("<i", len(b)) + b)


def test_fil_reads_reference_writer(hella):
    f = hella.Filterbank(GOLD / "ref_header.fil", 64)
    h = f.header
    assert (h.nchans, h.nbits, h.nifs, h.ibeam, h.nbeams, h.telescope_id, h.data_type) == (64, 8, 1, 3, 8, 7, 1)
    assert (h.fch1, h.foff, h.tsamp, h.tstart) == (468.75, -93.75 / 64, 1.048576e-3, 60000.25)
    assert h.source_name == b"FAKE_FRB" and h.rawdatafile == b"fixture.fil"
    size = (GOLD / "ref_header.fil").stat().st_size
    assert h.header_bytes == size - 16 * 64
    data = f.read(100)
    want = (np.arange(16 * 64, dtype=np.int64) * 37 % 251).astype(np.uint8).reshape(16, 64)
    assert np.array_equal(data, want)
    assert len(f.read(4)) == 0


def test_fil_checks(hella, tmp_path):
    def write(name, keys, body=b""):
        p = tmp_path / name
        with open(p, "wb") as fh:
            _w(fh, "HEADER_START")
            for k, fmt, v in keys:
                _w(fh, k)
                if fmt is None:
                    continue
                if fmt == "s":
                    _w(fh, v)
                else:
                    fh.write(struct.pack("<" + fmt, v))
            _w(fh, "HEADER_END")
            fh.write(body)
        return p

    base = [("nchans", "i", 32), ("nbits", "i", 8), ("tsamp", "d", 1e-3), ("signed", "b", 1), ("npuls", "q", 5),
            ("refdm", "d", 12.5)]
    f = hella.Filterbank(write("ok.fil", base, bytes(64)), 32)
    assert f.header.refdm == 12.5 and f.header.npuls == 5 and f.header.isign == b"\x01"
    assert f.read(10).shape == (2, 32)
    with pytest.raises(hella.HellaError):
        hella.Filterbank(write("nch.fil", base), 64)                       # NCHAN mismatch
    with pytest.raises(hella.HellaError):
        hella.Filterbank(write("bits.fil", [("nchans", "i", 32), ("nbits", "i", 16)]), 32)
    with pytest.raises(hella.HellaError):
        hella.Filterbank(write("key.fil", base + [("bogus_key", "i", 1)]), 32)
    p = tmp_path / "nohdr.fil"
    p.write_bytes(struct.pack("<i", 3) + b"abc" + bytes(16))
    with pytest.raises(hella.HellaError):
        hella.Filterbank(p, 32)
    # a frequency table: the fchannel values are kept in file order, fch1 = foff = 0 (sigproc.cpp:121-123)
    freqs = [468.75 - 1.5 * i for i in range(32)]
    tab = base + [("FREQUENCY_START", None, None)] + [("fchannel", "d", v) for v in freqs] + \
        [("FREQUENCY_END", None, None)]
    f = hella.Filterbank(write("tab.fil", tab, bytes(32)), 32)
    assert f.header.nfreq == 32 and (f.header.fch1, f.header.foff) == (0.0, 0.0)
    assert list(f.header.frequency_table[:32]) == freqs
    with pytest.raises(hella.HellaError):  # more entries than the table holds
        hella.Filterbank(write("bigtab.fil", [("fchannel", "d", 400.0)] * 4097 + base), 32)
    t = tmp_path / "trunc.fil"
    t.write_bytes(write("full.fil", base).read_bytes()[:30])
    with pytest.raises(hella.HellaError):
        hella.Filterbank(t, 32)


def _cands(n, seed=0):
    rng = np.random.default_rng(seed)
    c = np.zeros(n, hella_dtype())
    c["beam"] = rng.integers(0, 3, n)
    c["dm_idx"] = rng.integers(0, 50, n)
    c["width"] = rng.integers(0, 6, n)
    c["samp"] = rng.integers(0, 5000, n)
    c["snr"] = rng.uniform(6, 40, n).astype(np.float32)
    return c


def hella_dtype():
    import hella_gb300
    return hella_gb300.CAND_DTYPE


def _line(c, samp0, dms, tres):
    s = int(c["samp"]) + samp0
    return "%g %d %g %d %d %g %d\n" % (float(c["snr"]), s, tres * s / 86400.0, c["width"], c["dm_idx"],
                                        float(dms[c["dm_idx"]]), c["beam"])


def test_candidate_formats(hella, tmp_path):
    c = _cands(7)
    dms = np.linspace(0, 500, 50).astype(np.float32)
    text = hella.cands_format(c, 16384, dms, 1.0e-3)
    assert text == "".join(_line(x, 16384, dms, 1.0e-3) for x in c)
    path = tmp_path / "cands.txt"
    hella.cands_append(path, c[:3], 0, dms)
    hella.cands_append(path, c[3:], 0, dms)
    lines = path.read_text().splitlines()
    assert lines[0] == "SNR SAMP_START TIME_START WIDTH DM_IDX DM BEAM_IDX" and len(lines) == 8
    msg = hella.cands_coincidencer(5, c[:2], 100, dms, utc_start="2020-01-01-00:00:00", picoseconds=0, tsamp=1000)
    assert msg.splitlines()[0] == "5 2020-01-01-00:00:00 0 1000"
    assert msg.splitlines()[1:] == [l.rstrip("\n") for l in (_line(x, 100, dms, 1e-3) for x in c[:2])]
    assert hella.cands_coincidencer(2, c[:0], 0, dms) == "2\n"


def _listen():
    import socket

    srv = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
    srv.bind(("127.0.0.1", 0))
    srv.listen(1)
    return srv


def test_coincidencer_message_over_tcp(hella):
    """The message arrives whole on one connection, which is then closed
    (output_peaks' socket branch)."""
    c = _cands(600)
    dms = np.linspace(0, 500, 50).astype(np.float32)
    msg = hella.cands_coincidencer(9, c, 1000, dms)
    srv = _listen()
    got = []

    def serve():
        conn, _ = srv.accept()
        with conn:
            buf = b""
            while True:
                part = conn.recv(65536)
                if not part:
                    break
                buf += part
        got.append(buf)

    th = threading.Thread(target=serve)
    th.start()
    hella.cands_send("127.0.0.1", srv.getsockname()[1], msg, timeout_ms=5000)
    th.join(timeout=10)
    srv.close()
    assert got == [msg.encode()]
    assert len(msg) > 16384  # more than one small write's worth


def test_coincidencer_send_errors(hella):
    srv = _listen()
    port = srv.getsockname()[1]
    srv.close()  # nothing listens there now: connection refused
    with pytest.raises(hella.HellaError, match="socket"):
        hella.cands_send("127.0.0.1", port, "1\n", timeout_ms=2000)
    with pytest.raises(hella.HellaError, match="invalid"):
        hella.cands_send("not-an-address", 5000, "1\n")
    with pytest.raises(hella.HellaError, match="invalid"):
        hella.cands_send("127.0.0.1", 0, "1\n")


def _fof(c, dsamp, ddm, dw):
    n = len(c)
    parent = list(range(n))

    def root(i):
        while parent[i] != i:
            i = parent[i]
        return i

    for i in range(n):
        for j in range(i + 1, n):
            if (c[i]["beam"] == c[j]["beam"] and abs(int(c[i]["samp"]) - int(c[j]["samp"])) <= dsamp
                    and abs(int(c[i]["dm_idx"]) - int(c[j]["dm_idx"])) <= ddm
                    and abs(int(c[i]["width"]) - int(c[j]["width"])) <= dw):
                a, b = root(i), root(j)
                if a != b:
                    parent[max(a, b)] = min(a, b)
    return [root(i) for i in range(n)]


@pytest.mark.parametrize("n,seed", [(0, 0), (1, 1), (300, 2), (2000, 3)])
def test_cluster_matches_brute_force(hella, n, seed):
    c = _cands(n, seed)
    rep, lab = hella.cluster(c, 20, 3, 1)
    roots = _fof(c, 20, 3, 1)
    # same partition
    for i in range(n):
        for j in range(i + 1, min(n, i + 40)):
            assert (roots[i] == roots[j]) == (lab[i] == lab[j])
    assert len(rep) == len(set(roots))
    for k in range(len(rep)):
        members = c[lab == k]
        assert rep[k]["snr"] == members["snr"].max()


def test_flagstats(hella, tmp_path):
    fs = hella.FlagStats(4, 1000)
    cum = np.zeros(4, np.float32)
    want = np.zeros(4, np.int64)
    rng = np.random.default_rng(3)
    for _ in range(5):
        inc = rng.uniform(0, 0.2, 4).astype(np.float32)
        new = (cum + inc).astype(np.float32)
        want += (1000.0 * (new.astype(np.float64) - cum)).astype(np.int64)
        cum = new
        fs.update(cum)
    assert np.array_equal(fs.counts(), want)
    fs.append(tmp_path / "spec.txt")
    assert [int(x) for x in (tmp_path / "spec.txt").read_text().split()] == list(want)


def test_ring_in_order_with_header(hella):
    r = hella.Ring(64, 3)
    blocks = [bytes([i]) * (1 + i % 64) for i in range(50)]

    def produce():
        r.write_header("UTC_START 2025-01-01-00:00:00\nTSAMP 1048.576\n")
        for b in blocks:
            r.write(b, timeout_ms=5000)
        r.end()

    th = threading.Thread(target=produce)
    th.start()
    assert hella.header_get(r.read_header(5000), "TSAMP") == "1048.576"
    got = []
    while (b := r.read(timeout_ms=5000)) is not None:
        got.append(b)
    th.join()
    assert got == blocks


def test_ring_timeouts(hella):
    r = hella.Ring(16, 2)
    with pytest.raises(hella.HellaError, match="timed out"):
        r.read(timeout_ms=20)
    r.write(b"a")
    r.write(b"b")
    with pytest.raises(hella.HellaError, match="timed out"):
        r.write(b"c", timeout_ms=20)            # both blocks full
    assert r.read() == b"a"


def test_dada_header_from_reference_converter(hella):
    text = (GOLD / "ref_dada_header.txt").read_text()
    assert hella.header_get(text, "UTC_START") == "2020-01-01-00:00:00"
    assert hella.header_get(text, "TSAMP") == "1000"
    assert hella.header_get(text, "NBIT") == "16"
    assert hella.header_get(text, "PICOSECONDS") == "0"
    assert hella.header_get(text, "MISSING") is None
    assert hella.header_get("A 1\nA 2\n", "A") == "2"                 # later lines win
    assert hella.header_get("A 1\nBROKEN\nB 2\n", "B") is None         # an invalid line ends the parse
    assert hella.header_get("A   spaced value\n", "A") == "spaced value"
