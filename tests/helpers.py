"""Shared helpers for the tests: parameter plumbing between the product's
C-ABI parameters and the oracle pipeline."""
import numpy as np


def oracle_pipeline(oracle, params: dict, **over):
    return oracle.Pipeline.from_params(params, **over)


def small_params(**over):
    """A small search that the oracle finishes in well under a second."""
    p = dict(nchan=128, nbeam=1, gulp=2048, tsamp=1.048576e-3, plan_dt=1.048576e-3, f0_mhz=468.75,
             df_mhz=-(468.75 - 375.0) / 128, dm_min=0.0, dm_max=120.0, dm_tol=1.25, ti_us=500.0,
             width_min=1, width_max=16, snr=6.0)
    p.update(over)
    return p


def cands_equal(a: np.ndarray, b: np.ndarray) -> bool:
    if len(a) != len(b):
        return False
    for k in ("beam", "dm_idx", "width", "samp"):
        if not np.array_equal(a[k], b[k]):
            return False
    return np.array_equal(a["snr"].view(np.uint32), b["snr"].view(np.uint32))
