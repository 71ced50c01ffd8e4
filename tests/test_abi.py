"""The C-ABI boundary without a GPU: the library loads, exports every
function include/*.h declares, its host-side plan math equals the oracle's
bit for bit, and argument errors come back as status codes."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b((?:hdd|hella)_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_symbol(hella):
    out = subprocess.run(["nm", "-D", "--defined-only", str(hella.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    assert len(declared_functions()) > 40


def test_plan_math_matches_oracle(hella, oracle):
    """hdd_create_plan + hdd_generate_dm_list (host only) against the oracle."""
    for nchan, dt, dm_max, ti, tol in [(512, 1.048576e-3, 500.0, 500.0, 1.25), (2048, 0.524288e-3, 2000.0, 40.0, 1.25),
                                       (3072, 1e-3, 1000.0, 40.0, 1.3)]:
        f0 = 468.75
        df = -(f0 - 375.0) / nchan if nchan != 3072 else -0.03075
        plan = hella.Plan(nchan, dt, f0, df)
        plan.generate_dm_list(0.0, dm_max, ti, tol)
        f32 = lambda v: float(np.float32(v))
        dms = oracle.dm_list(0.0, f32(dm_max), f32(ti), f32(tol), nchan, f32(dt), f32(f0), f32(df))
        assert np.array_equal(plan.dm_list().view(np.uint32), dms.view(np.uint32))
        delays = oracle.dm_delays(dms, oracle.delay_table(nchan, f32(dt), f32(f0), f32(df)))
        assert np.array_equal(plan.delay_table(), delays)
        assert plan.max_delay == delays[-1, -1]
        plan.close()


def test_plan_error_codes(hella):
    L = hella.lib()
    h = C.c_void_p()
    assert L.hdd_create_plan(C.byref(h), 0, 1e-3, 468.75, -0.1) == 3  # nchans exceeds limit
    assert L.hdd_create_plan(C.byref(h), 64, 1e-3, 468.75, -0.5) == 0
    buf = np.zeros(16, np.uint8)
    # no DM list yet
    assert L.hdd_execute(h, 10, buf.ctypes.data, 8, buf.ctypes.data, 32, 0) in (7, 8)
    L.hdd_generate_dm_list(h, 0.0, 50.0, 40.0, 1.3)
    md = L.hdd_get_max_delay(h)
    assert L.hdd_execute_adv(h, md, buf.ctypes.data, 8, 64, buf.ctypes.data, 32, 4, 0) == 8  # too few nsamps
    assert L.hdd_execute_adv(h, md + 10, buf.ctypes.data, 4, 64, buf.ctypes.data, 32, 40, 0) == 10
    assert L.hdd_execute_adv(h, md + 10, buf.ctypes.data, 8, 64, buf.ctypes.data, 16, 40, 0) == 11
    assert L.hdd_execute_adv(h, md + 10, buf.ctypes.data, 8, 32, buf.ctypes.data, 32, 40, 0) == 6
    assert L.hdd_execute_adv(h, md + 10, buf.ctypes.data, 8, 64, buf.ctypes.data, 32, 39, 0) == 6
    assert L.hdd_execute_adv(h, md + 10, buf.ctypes.data, 8, 64, buf.ctypes.data, 32, 40,
                             hella.HDD_HOST_POINTERS | hella.HDD_DEVICE_POINTERS) == 9
    assert L.hdd_get_error_string(6) == b"invalid stride"
    L.hdd_destroy_plan(h)


def test_plan_rejects_dm_lists_the_kernels_cannot_serve(hella):
    """Negative, NaN, infinite or int-overflowing trials come back as
    HDD_UNKNOWN_ERROR and leave the plan's list as it was; any order of
    valid trials is accepted, with max_delay the largest delay of all."""
    unknown = 16
    plan = hella.Plan(128, 1e-3, 468.75, -0.5)
    plan.generate_dm_list(0.0, 50.0, 40.0, 1.3)
    n0, md0 = plan.dm_count, plan.max_delay
    L = hella.lib()
    for bad in ([5.0, -1.0], [float("nan")], [float("inf")], [1e12], [3.0e38]):
        a = np.asarray(bad, np.float32)
        assert L.hdd_set_dm_list(plan.h, a.ctypes.data, a.size) == unknown, bad
        assert (plan.dm_count, plan.max_delay) == (n0, md0)
    for args in ((-1.0, 50.0, 40.0, 1.3), (0.0, float("nan"), 40.0, 1.3), (0.0, 50.0, 40.0, 1.0),
                 (0.0, 1e12, 40.0, 1.3)):
        assert L.hdd_generate_dm_list(plan.h, *args) == unknown, args
        assert (plan.dm_count, plan.max_delay) == (n0, md0)
    plan.generate_dm_list(30.0, 10.0, 40.0, 1.3)  # end below start: the single trial 30
    assert list(plan.dm_list()) == [30.0]
    plan.set_dm_list(np.asarray([50.0, 0.0, 20.0], np.float32))
    d = plan.delay_table()
    assert plan.max_delay == d.max() == d[0, -1]
    plan.close()


def test_search_rejects_bad_params(hella):
    L = hella.lib()
    h = C.c_void_p()
    for bad in (dict(nchan=100), dict(gulp=100), dict(width_max=1), dict(dm_tol=1.0), dict(smooth_anchor=3),
                dict(bp_median=0), dict(bp_median=4), dict(bp_median=65), dict(nchan=32, bp_median=33),
                dict(always_find_peaks=2)):
        p = hella.default_params(**bad)
        assert L.hella_create(C.byref(h), C.byref(p)) == 1
    assert L.hella_status_string(6) == b"hbm budget exceeded"


def test_batch_bytes_sizing(hella):
    """hella_batch_bytes (host only): affine in the number of slots, each slot
    holding at least its ring (5 bytes per channel-sample), its dedispersed
    plane and its tile tables (6 bytes per trial and channel); per-beam DM
    ceilings shrink it; a batch without beams is refused."""
    p = dict(nchan=128, gulp=2048, tsamp=1.048576e-3, plan_dt=1.048576e-3, f0_mhz=468.75,
             df_mhz=-(468.75 - 375.0) / 128, dm_min=0.0, dm_max=400.0, dm_tol=1.25, ti_us=40.0,
             width_min=1, width_max=64, snr=7.0)
    kw = dict(dynamic=True, inflight=2, widths_per_pass=6)
    size = {n: hella.batch_bytes(hella.default_params(**dict(p, nbeam=n)), **kw) for n in (3, 4, 5)}
    step = size[4] - size[3]
    assert size[5] - size[4] == step
    plan = hella.Plan(p["nchan"], p["plan_dt"], p["f0_mhz"], p["df_mhz"])
    plan.generate_dm_list(p["dm_min"], p["dm_max"], p["ti_us"], p["dm_tol"])
    ndms, nch = plan.dm_count, p["nchan"]
    ntime = 32 * ((p["gulp"] + plan.max_delay + p["width_max"]) // 32 + 1)
    plan.close()
    assert step >= nch * ntime * 5 + ndms * (p["gulp"] + p["width_max"]) * 4 + (ndms + 15) * nch * 6
    lower = hella.batch_bytes(hella.default_params(**dict(p, nbeam=4)), dm_max=np.full(4, 150.0, np.float32),
                              inflight=2, widths_per_pass=6)
    assert lower < size[4]
    with pytest.raises(hella.HellaError):
        hella.batch_bytes(hella.default_params(**dict(p, nbeam=0)), **kw)
