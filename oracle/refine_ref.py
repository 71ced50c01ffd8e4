"""FP64 reference of the candidate-refinement model -- test infrastructure.

This is the oracle of the GB300 refinement kernels (include/hella_refine.h),
used only by the tests and the benchmark's CPU baseline.  The refinement has
no counterpart in casm-hella, whose search stops at the detection grid
(src/hella/src/peaks.cu:31-117 reports a DM trial, a boxcar width and a
sample), so nothing here restates reference code: it states the model in
double precision.

Cutout i: fp32 [nchan][nsamp], channel c shifted by the integer delay of the
detection DM dm_ref: off_c = (int)(fp32(dm_ref * tab_c) + 0.5f), tab_c the
per-unit-DM delay table of the dedispersion plan (4.148808e3 s MHz^2 *
(1/f_c^2 - 1/f0^2) / tsamp, stored in fp32).  Model:
    m[c][t] = amp * (f_c/f0)^index * exp(-u^2/2),  u = (t - mu_c)/sigma,
    mu_c = t0 + dm * tab_c - off_c,  sigma = width_ms / (2 sqrt(2 ln 2) tsamp_ms),
    chi2 = sum (d - m)^2.
theta = (dm, t0, width_ms, amp, index).
"""
from __future__ import annotations

import math

import numpy as np

FWHM = 2.0 * math.sqrt(2.0 * math.log(2.0))


def delay_table(nchan: int, tsamp: float, f0: float, df: float) -> np.ndarray:
    """fp32 samples of delay per unit DM, as the plan stores them."""
    fc = f0 - np.arange(nchan, dtype=np.float64) * abs(df)
    return (4.148808e3 / tsamp * (1.0 / (fc * fc) - 1.0 / (f0 * f0))).astype(np.float32)


def log_freq(nchan: int, f0: float, df: float) -> np.ndarray:
    fc = f0 - np.arange(nchan, dtype=np.float64) * abs(df)
    return np.log(fc / f0).astype(np.float32)


def offsets(dm_ref: float, tab: np.ndarray) -> np.ndarray:
    """The plan's integer delays of the detection DM (fp32 arithmetic)."""
    p = np.float32(dm_ref) * tab.astype(np.float32)
    return (p + np.float32(0.5)).astype(np.int64)


class Geometry:
    def __init__(self, nchan: int, nsamp: int, tsamp: float, f0: float, df: float):
        self.nchan, self.nsamp, self.tsamp = nchan, nsamp, tsamp
        self.tab = delay_table(nchan, tsamp, f0, df).astype(np.float64)
        self.lnf = log_freq(nchan, f0, df).astype(np.float64)
        self.c_w = 1.0 / (FWHM * tsamp * 1e3)

    def parts(self, theta, dm_ref):
        dm, t0, w, amp, idx = (float(v) for v in theta)
        off = offsets(dm_ref, self.tab.astype(np.float32)).astype(np.float64)
        mu = t0 + dm * self.tab - off
        sigma = w * self.c_w
        t = np.arange(self.nsamp, dtype=np.float64)
        u = (t[None, :] - mu[:, None]) / sigma
        e = np.exp(-0.5 * u * u)
        s = np.exp(idx * self.lnf)
        return amp, s, sigma, u, e

    def model(self, theta, dm_ref) -> np.ndarray:
        amp, s, sigma, u, e = self.parts(theta, dm_ref)
        return amp * s[:, None] * e

    def chi2(self, d, theta, dm_ref) -> float:
        r = d.astype(np.float64) - self.model(theta, dm_ref)
        return float(np.sum(r * r))

    def grad(self, d, theta, dm_ref) -> np.ndarray:
        """Analytic d chi2 / d theta in FP64."""
        amp, s, sigma, u, e = self.parts(theta, dm_ref)
        m = amp * s[:, None] * e
        r = d.astype(np.float64) - m
        g_m = -2.0 * r
        dmu = np.sum(g_m * m * u / sigma, axis=1)        # per channel d chi2 / d mu_c
        return np.array([
            np.sum(dmu * self.tab),                       # dm
            np.sum(dmu),                                  # t0
            np.sum(g_m * m * u * u / sigma) * self.c_w,   # width (ms)
            np.sum(g_m * s[:, None] * e),                 # amp
            np.sum(g_m * m * self.lnf[:, None]),          # index
        ])

    def fd_grad(self, d, theta, dm_ref, rel: float = 1e-7) -> np.ndarray:
        """Central finite differences of chi2 in FP64."""
        theta = np.asarray(theta, dtype=np.float64)
        g = np.zeros(5)
        for k in range(5):
            h = rel * max(1.0, abs(theta[k]))
            tp, tm = theta.copy(), theta.copy()
            tp[k] += h
            tm[k] -= h
            g[k] = (self.chi2(d, tp, dm_ref) - self.chi2(d, tm, dm_ref)) / (2 * h)
        return g
