"""hdd_execute_noalloc: dedispersion for callers that cannot allocate device
memory while they run (a real-time loop that must not stall in the
allocator, code living inside another component's memory budget).  It must
give the same sums as hdd_execute_adv with device pointers, call after
call, although every call reuses one fixed scratch array.  Kept in a file
of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(hella, nchan=256, dm_max=150.0):
    plan = hella.Plan(nchan, 1e-3, 468.75, -(468.75 - 375.0) / nchan)
    plan.generate_dm_list(0.0, dm_max, 40.0, 1.25)
    return plan


def test_noalloc_matches_execute_adv_twice(hella):
    torch = pytest.importorskip("torch")
    L = hella.lib()
    plan = _plan(hella)
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    nsamps = plan.max_delay + 3000
    nout = nsamps - plan.max_delay
    rng = np.random.default_rng(99)
    for call in range(2):  # the second call must not see the first call's scratch
        x = torch.from_numpy(rng.integers(0, 256, (nsamps, plan.nchans), dtype=np.uint8)).cuda()
        ref = torch.empty((plan.dm_count, nout), dtype=torch.float32, device="cuda")
        got = torch.full((plan.dm_count, nout), -1.0, dtype=torch.float32, device="cuda")
        plan.execute_adv(nsamps, x, plan.nchans, ref, nout * 4, flags=hella.HDD_DEVICE_POINTERS)
        rc = L.hdd_execute_noalloc(plan.h, nsamps, x.data_ptr(), 8, plan.nchans, got.data_ptr(), 32, nout * 4,
                                   hella.HDD_DEVICE_POINTERS)
        assert rc == 0, hella.HDD_ERRORS[rc]
        torch.cuda.synchronize()
        # integer sums in fp32: the tolerance the parity tests use for them is exact equality
        assert torch.equal(got, ref), call
    plan.close()


def test_noalloc_rejects_oversize_and_host_pointers(hella):
    L = hella.lib()
    plan = _plan(hella, nchan=2048, dm_max=500.0)
    buf = np.zeros(64, np.uint8)
    nsamps = plan.max_delay + 8192  # 2048 x ~13k samples x 5 bytes > 32 MiB
    rc = L.hdd_execute_noalloc(plan.h, nsamps, buf.ctypes.data, 8, plan.nchans, buf.ctypes.data, 32,
                               (nsamps - plan.max_delay) * 4, hella.HDD_DEVICE_POINTERS)
    assert hella.HDD_ERRORS[rc] == "HDD_STATIC_SCRATCH_EXCEEDED"
    assert b"static scratch" in L.hdd_get_error_string(rc)
    rc = L.hdd_execute_noalloc(plan.h, plan.max_delay + 10, buf.ctypes.data, 8, plan.nchans, buf.ctypes.data,
                               32, 40, hella.HDD_HOST_POINTERS)
    assert hella.HDD_ERRORS[rc] == "HDD_INVALID_FLAG_COMBINATION"
    plan.close()
