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


def test_noalloc_matches_execute_adv_twice(hella, oracle):
    """Two calls in a row, each on new data, equal to hdd_execute_adv on the
    same device buffers and, as integer sums, to the oracle's brute force."""
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
        want = oracle.dedisperse(x.cpu().numpy(), plan.delay_table(), nout=nout)
        assert np.array_equal(got.cpu().numpy(), want), call
    plan.close()


def test_noalloc_leaves_device_memory_untouched(hella):
    """The property that defines the entry point: after a first call (which
    resolves the scratch address and loads the kernels), more calls with
    other sample counts, synchronous and HDD_ASYNC, change the free device
    memory by nothing."""
    torch = pytest.importorskip("torch")
    L = hella.lib()
    plan = _plan(hella)
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    sizes = [plan.max_delay + n for n in (3000, 1000, 4099, 257)]
    rng = np.random.default_rng(7)
    xs = [torch.from_numpy(rng.integers(0, 256, (n, plan.nchans), dtype=np.uint8)).cuda() for n in sizes]
    outs = [torch.zeros((plan.dm_count, n - plan.max_delay), dtype=torch.float32, device="cuda") for n in sizes]

    def call(i, flags):
        n = sizes[i]
        return L.hdd_execute_noalloc(plan.h, n, xs[i].data_ptr(), 8, plan.nchans, outs[i].data_ptr(), 32,
                                     (n - plan.max_delay) * 4, flags)

    assert call(0, hella.HDD_DEVICE_POINTERS) == 0  # warm-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for i in (1, 2, 3, 0):
        assert call(i, hella.HDD_DEVICE_POINTERS | hella.HDD_ASYNC) == 0
        assert call(i, hella.HDD_DEVICE_POINTERS) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
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
    # the transpose's grid limit is not a scratch limit: the code hdd_execute_guru gives it
    rc = L.hdd_execute_noalloc(plan.h, 65535 * 32 + 1, buf.ctypes.data, 8, plan.nchans, buf.ctypes.data,
                               32, 4 * (65535 * 32 + 1), hella.HDD_DEVICE_POINTERS)
    assert hella.HDD_ERRORS[rc] == "HDD_UNKNOWN_ERROR"
    plan.close()
