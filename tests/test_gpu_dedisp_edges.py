"""Known-answer and edge cases of the GPU dedispersion through the dedisp-shaped
C ABI: a single-channel impulse lands at its known delay, sample counts that
are not multiples of 4 (and one more than the maximum delay), every channel
killed, and the largest channel count the API accepts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(hella, nchan, dm_max, dt=1e-3):
    p = hella.Plan(nchan, dt, 468.75, -(468.75 - 375.0) / nchan)
    p.generate_dm_list(0.0, dm_max, 40.0, 1.25)
    return p


@pytest.mark.parametrize("chan", [0, 97, 255])
def test_impulse_lands_at_known_delay(hella, chan):
    plan = _plan(hella, 256, 300.0)
    delays = plan.delay_table()
    md = plan.max_delay
    nsamps = md + 2049
    x = np.zeros((nsamps, 256), np.uint8)
    s = md + 700
    x[s, chan] = 200
    out = plan.dedisperse(x)
    want = np.zeros_like(out)
    for d in range(plan.dm_count):
        t = s - delays[d, chan]
        if 0 <= t < out.shape[1]:
            want[d, t] = 200
    assert np.array_equal(out, want)


@pytest.mark.parametrize("extra", [1, 7, 1023, 4097])
def test_ragged_sample_counts(hella, oracle, extra):
    plan = _plan(hella, 192, 250.0)
    rng = np.random.default_rng(extra)
    x = rng.integers(0, 256, (plan.max_delay + extra, 192), dtype=np.uint8)
    got = plan.dedisperse(x)
    assert got.shape[1] == extra
    assert np.array_equal(got, oracle.dedisperse(x, plan.delay_table()))


def test_all_channels_killed(hella):
    plan = _plan(hella, 128, 200.0)
    plan.set_killmask(np.zeros(128, np.int32))
    x = np.full((plan.max_delay + 300, 128), 77, np.uint8)
    assert not plan.dedisperse(x).any()


def test_max_channels(hella, oracle):
    n = 16384  # HDD_MAX_NCHANS
    plan = _plan(hella, n, 12.0, dt=4e-3)
    rng = np.random.default_rng(5)
    x = rng.integers(0, 256, (plan.max_delay + 1500, n), dtype=np.uint8)
    got = plan.dedisperse(x)
    rows = np.unique(np.linspace(0, plan.dm_count - 1, 6).astype(int))
    want = oracle.dedisperse(x, plan.delay_table()[rows])
    assert np.array_equal(got[rows], want)
    with pytest.raises(hella.HellaError):
        hella.Plan(n + 1, 4e-3, 468.75, -0.005)
