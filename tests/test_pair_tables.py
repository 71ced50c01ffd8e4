"""The group-row tables of add modes 5 and 6 on the CPU (no GPU): the host
tables the plan builds (hdd_get_pair_tables) are walked the way
k_pair_build and k_pair_sum walk them -- rows built from a ring with a
window start anywhere, every stage's row copies staged, every trial's
words read at its offset -- and the sums must equal the oracle's
channel-by-channel dedispersion bit for bit, with every copy inside its
row and every read inside its stage.  Cases: killmasks leaving odd counts
and short last groups, a single active channel, non-adjacent groups,
ascending-frequency bands (negative relative delays), sub-ranges of
trials, both stage widths and both group sizes."""
import numpy as np
import pytest

DPT, RMAX = 16, 32


def emulate(T, x_ring, win0, nout, ndm):
    """Sums of trials [0, ndm) of the tables over window start win0."""
    cc, ntt = T["stage_groups"], T["time_tiles"]
    R = x_ring.shape[1]
    rows = np.zeros(T["words"], np.int64)
    roff, rw = T["roff"], T["rwords"].astype(np.int64)
    assert np.all(roff % 4 == 0) and np.all(rw % 4 == 0) and roff[-1] + rw[-1] == T["words"]
    for k in range(T["ngroups"]):
        for r in range(T["prow"][k], T["prow"][k + 1]):
            c0, c1, r1, first = T["rinfo"][r]
            c2, c3, r2, r3 = T["rinfo2"][r]
            stride = T["rtile"][r]
            i = np.arange(rw[r])
            p = first + (i // stride) * 1024 + i % stride  # position of word i
            lo = x_ring[c0, (win0 + p) % R].copy()
            hi = x_ring[c0, (win0 + p + 512) % R].copy()
            for i, (c, rel) in enumerate(((c1, r1), (c2, r2), (c3, r3))):
                if c < 0:
                    continue
                assert T["prange"][k, i, 0] <= rel <= T["prange"][k, i, 1]
                lo += x_ring[c, (win0 + p + rel) % R]
                hi += x_ring[c, (win0 + p + rel + 512) % R]
            assert lo.max() < 1 << 16 and hi.max() < 1 << 16
            rows[roff[r]: roff[r] + rw[r]] = lo | (hi << 16)
    rec = T["rec"].astype(np.int64)
    out = np.zeros((ndm, ntt * 1024), np.int64)
    rows0 = 4 + cc * DPT
    assert T["tile_st"][0] == 0 and T["tile_st"][-1] == rec.shape[0]
    for t in range(T["ntiles"]):
        for tt in range(ntt):
            t0 = tt * 1024
            tot = np.zeros((DPT, 1024), np.int64)
            for s in range(T["tile_st"][t], T["tile_st"][t + 1]):
                r = rec[s]
                ng, nr = int(r[0]), int(r[1])
                assert 1 <= ng <= cc and 1 <= nr <= RMAX
                buf = []
                for j in range(nr):
                    lo, hi, packed, stride = r[rows0 + 4 * j: rows0 + 4 * j + 4]
                    start = (lo & 0xffffffff) | (hi << 32)
                    nw, slot = packed & 0xffff, (packed >> 16) * 16
                    u = np.searchsorted(roff, start, side="right") - 1
                    assert stride == T["rtile"][u] and (stride == 1024 or nw <= stride)
                    assert start % 4 == 0 and nw % 4 == 0 and slot == 4 * sum(len(b) for b in buf)
                    assert start + (ntt - 1) * stride + nw <= roff[u] + rw[u]  # inside the row, last tile too
                    assert start - roff[u] + nw <= stride or stride == 1024   # inside its tile's window
                    buf.append(rows[start + tt * stride: start + tt * stride + nw])
                buf = np.concatenate(buf)
                assert buf.size * 4 <= T["max_stage_bytes"] or ng == 1
                for i in range(ng):
                    for m in range(DPT):
                        o = int(r[4 + i * DPT + m])
                        assert o % 4 == 0 and 0 <= o and o // 4 + 511 < buf.size
                        wa, wb = buf[o // 4: o // 4 + 256], buf[o // 4 + 256: o // 4 + 512]
                        tot[m, 0:256] += wa & 0xffff
                        tot[m, 512:768] += wa >> 16
                        tot[m, 256:512] += wb & 0xffff
                        tot[m, 768:1024] += wb >> 16
            for m in range(DPT):
                d = t * DPT + m
                if d < ndm:
                    out[d, t0:t0 + 1024] = tot[m]
    return out[:, :nout]


CASES = [  # nchan, dm_max, killmask kind, ascending band, first, count
    (32, 300.0, "none", False, 0, None),
    (40, 500.0, "odd", False, 0, None),
    (64, 800.0, "runs", True, 0, None),
    (24, 200.0, "one", False, 0, None),
    (48, 400.0, "none", False, 9, 23),
]


@pytest.mark.parametrize("channels,stage_groups", [(2, 4), (2, 8), (4, 4), (4, 8)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_pair_tables_sum_like_the_oracle(hella, oracle, channels, stage_groups, case):
    nch, dm_max, kind, asc, first, count = CASES[case]
    f0 = 375.0 if asc else 468.75
    df = (1 if asc else -1) * (468.75 - 375.0) / nch
    plan = hella.Plan(nch, 1e-3, f0, df)
    plan.generate_dm_list(0.0, dm_max, 40.0, 1.25)
    rng = np.random.default_rng(case * 10 + channels + stage_groups)
    km = np.ones(nch, np.int32)
    if kind == "odd":
        km[rng.choice(nch, 5, replace=False)] = 0
    elif kind == "runs":
        km[10:21] = 0
        km[rng.choice(nch, 7, replace=False)] = 0
    elif kind == "one":
        km[:] = 0
        km[7] = 1
    plan.set_killmask(km)
    ndm = plan.dm_count - first if count is None else count
    nout = 1500 + 37 * case
    ntt = -(-nout // 1024)
    T = plan.pair_tables(first, ndm, channels, stage_groups, ntt)
    delays = plan.delay_table()[first:first + ndm]
    md = int(plan.max_delay)
    R = (nout + md + 700) // 4 * 4
    x = rng.integers(0, 256, (nch, R))
    win0 = int(rng.integers(0, R))
    got = emulate(T, x, win0, nout, ndm)
    window = x[:, (win0 + np.arange(nout + md)) % R].T.astype(np.uint8)  # [nsamps][nchan]
    want = oracle.dedisperse(window, delays, killmask=km, nout=nout)
    assert np.array_equal(got, want.astype(np.int64))
    plan.close()


def test_pair_tables_long_rows(hella, oracle):
    """512 channels, DM 0-300: adjacent channels keep one relative delay
    over hundreds of trials, so some pair rows are read over more than a
    tile's width and are kept as one run (words per tile 1024), the rest in
    per-tile windows; both kinds in one set of tables."""
    nch = 512
    plan = hella.Plan(nch, 1e-3, 468.75, -(468.75 - 375.0) / nch)
    plan.generate_dm_list(0.0, 300.0, 40.0, 1.25)
    nout, ndm = 1600, plan.dm_count
    T = plan.pair_tables(0, ndm, 2, 8, 2)
    assert (T["rtile"] == 1024).sum() > 100 and (T["rtile"] < 1024).sum() > 100
    rng = np.random.default_rng(7)
    md = int(plan.max_delay)
    R = (nout + md + 700) // 4 * 4
    x = rng.integers(0, 256, (nch, R))
    win0 = int(rng.integers(0, R))
    got = emulate(T, x, win0, nout, ndm)
    window = x[:, (win0 + np.arange(nout + md)) % R].T.astype(np.uint8)
    assert np.array_equal(got, oracle.dedisperse(window, plan.delay_table(), nout=nout).astype(np.int64))
    plan.close()


def test_pair_tables_reject_bad_shapes(hella):
    plan = hella.Plan(32, 1e-3, 468.75, -0.1)
    plan.generate_dm_list(0.0, 100.0, 40.0, 1.25)
    for args in ((0, 4, 3, 4, 2), (0, 4, 2, 6, 2), (0, 4, 2, 4, 0), (0, 0, 2, 4, 2), (plan.dm_count, 1, 2, 4, 2)):
        with pytest.raises(hella.HellaError):
            plan.pair_tables(*args)
    plan.close()
