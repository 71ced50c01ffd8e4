"""Seeded synthetic filterbank gulps for the search's parity tests and bench.

No public dataset is named for this path; these generators stand in for it
with the shapes and value distributions of the search configurations:
u8 samples ~ round(N(mean, sd)) clipped to 0..255, narrowband RFI channels
with a larger sd, broadband impulses, and dispersed Gaussian bursts.  The
dispersion follows the reference's injection script
(scripts/make_noise_fil_with_frb.py:123-173): per-channel delay
4.148808 ms DM (f_GHz^-2 - f0_GHz^-2) rounded to whole samples, a Gaussian
pulse painted within +-4 sigma of each channel's arrival.  Every gulp is a
pure function of (seed, gulp index), so a stream can be regenerated
anywhere, and bursts that straddle gulps are painted consistently.
"""
from __future__ import annotations

import dataclasses as dc
import math

import numpy as np

K_MS = 4.148808  # ms GHz^2 / (pc cm^-3)


@dc.dataclass
class Burst:
    t0: int            # absolute arrival sample at channel 0 (f0)
    dm: float
    fwhm_ms: float
    amp: float         # counts per channel at f0 (before the spectral index)
    index: float = 0.0


@dc.dataclass
class Spike:
    t0: int            # absolute first sample
    width: int         # samples
    amp: float         # counts, all channels


@dc.dataclass
class Sky:
    nchan: int
    tsamp: float       # s
    f0: float          # MHz, channel 0
    df: float          # MHz per channel (negative: descending)
    seed: int
    mean: float = 128.0
    sd: float = 20.0
    rfi_chans: tuple = ()
    rfi_sd: float = 80.0
    slope: float = 0.0              # bandpass gain 1 + slope*(c/(nchan-1) - 0.5)
    bursts: list = dc.field(default_factory=list)
    spikes: list = dc.field(default_factory=list)

    def freqs(self) -> np.ndarray:
        return self.f0 + np.arange(self.nchan) * self.df

    def delays(self, dm: float) -> np.ndarray:
        f = self.freqs() / 1000.0
        ms = K_MS * dm * (1.0 / f**2 - 1.0 / (self.f0 / 1000.0) ** 2)
        return np.round(ms / (self.tsamp * 1000.0)).astype(np.int64)

    def gulp(self, g: int, n: int) -> np.ndarray:
        """Samples [g*n, (g+1)*n) as u8 [n][nchan]."""
        rng = np.random.Generator(np.random.PCG64([self.seed, g]))
        x = rng.standard_normal((n, self.nchan), dtype=np.float32)
        sd = np.full(self.nchan, self.sd, np.float32)
        if len(self.rfi_chans):
            sd[list(self.rfi_chans)] = self.rfi_sd
        gain = 1.0 + self.slope * (np.arange(self.nchan, dtype=np.float32) / max(1, self.nchan - 1) - 0.5)
        x *= sd
        x += (self.mean * gain).astype(np.float32)
        a0 = g * n
        for s in self.spikes:
            lo, hi = max(s.t0, a0), min(s.t0 + s.width, a0 + n)
            if lo < hi:
                x[lo - a0:hi - a0] += s.amp
        f = self.freqs()
        for b in self.bursts:
            dl = self.delays(b.dm)
            sig = max(1.0, b.fwhm_ms / 2.3548 / (self.tsamp * 1000.0))
            hw = int(math.ceil(4.0 * sig))
            centers = b.t0 + dl
            sel = np.nonzero((centers + hw >= a0) & (centers - hw < a0 + n))[0]
            if sel.size == 0:
                continue
            spec = b.amp * (f[sel] / self.f0) ** b.index
            offs = np.arange(-hw, hw + 1)
            prof = np.exp(-0.5 * (offs / sig) ** 2)
            tt = centers[sel][:, None] + offs[None, :] - a0
            ok = (tt >= 0) & (tt < n)
            cc = np.broadcast_to(sel[:, None], tt.shape)
            np.add.at(x, (tt[ok], cc[ok]), (spec[:, None] * prof[None, :])[ok].astype(np.float32))
        np.rint(x, out=x)
        np.clip(x, 0, 255, out=x)
        return x.astype(np.uint8)


def gulp_device(sky: Sky, g: int, n: int, out=None):
    """Samples [g*n, (g+1)*n) of `sky` as a u8 [n][nchan] CUDA tensor (into
    `out` if given): the model of Sky.gulp drawn on the GPU with torch's
    generator, for workloads too large to draw on the host.  Same
    distribution, different random stream from Sky.gulp."""
    import torch

    gen = torch.Generator(device="cuda")
    gen.manual_seed((sky.seed * 1000003 + g) & 0x7FFFFFFFFFFFFFFF)
    x = torch.randn((n, sky.nchan), generator=gen, device="cuda", dtype=torch.float32)
    sd = torch.full((sky.nchan,), sky.sd, device="cuda")
    if len(sky.rfi_chans):
        sd[list(sky.rfi_chans)] = sky.rfi_sd
    c = torch.arange(sky.nchan, device="cuda", dtype=torch.float32)
    gain = 1.0 + sky.slope * (c / max(1, sky.nchan - 1) - 0.5)
    x.mul_(sd).add_(sky.mean * gain)
    a0 = g * n
    for sp in sky.spikes:
        lo, hi = max(sp.t0, a0), min(sp.t0 + sp.width, a0 + n)
        if lo < hi:
            x[lo - a0:hi - a0] += sp.amp
    f = sky.freqs()
    for b in sky.bursts:
        dl = sky.delays(b.dm)
        sig = max(1.0, b.fwhm_ms / 2.3548 / (sky.tsamp * 1000.0))
        hw = int(math.ceil(4.0 * sig))
        centers = b.t0 + dl
        sel = np.nonzero((centers + hw >= a0) & (centers - hw < a0 + n))[0]
        if sel.size == 0:
            continue
        spec = b.amp * (f[sel] / sky.f0) ** b.index
        offs = np.arange(-hw, hw + 1)
        prof = np.exp(-0.5 * (offs / sig) ** 2)
        tt = centers[sel][:, None] + offs[None, :] - a0
        ok = (tt >= 0) & (tt < n)
        cc = np.broadcast_to(sel[:, None], tt.shape)
        vals = (spec[:, None] * prof[None, :])[ok].astype(np.float32)
        x.index_put_((torch.from_numpy(tt[ok]).cuda(), torch.from_numpy(np.ascontiguousarray(cc[ok])).cuda()),
                     torch.from_numpy(vals).cuda(), accumulate=True)
    x.round_().clamp_(0, 255)
    if out is None:
        return x.to(torch.uint8)
    out.copy_(x)
    return out


def snr_amp(snr: float, sd: float, nchan: int, fwhm_ms: float, tsamp: float) -> float:
    """Per-channel amplitude of a flat-spectrum Gaussian with band-integrated
    matched-filter S/N `snr` in noise of `sd` counts."""
    sig = max(1.0, fwhm_ms / 2.3548 / (tsamp * 1000.0))
    return snr * sd / math.sqrt(nchan * sig * math.sqrt(math.pi))


# ------------------------------------------------------------ configurations
F0, FLO = 468.75, 375.0


def first_window(sky: Sky, gulp: int, dm_max: float, wmax: int):
    """(gulp index, first absolute sample, NTIME) of the first searched
    window, from the search geometry (casm_hella_refactored.cu:217-224,632):
    NTIME = 32*((gulp + max_delay + wmax)//32 + 1), searched from gulp
    NTIME//gulp on, window = the last NTIME samples of that gulp."""
    md = int(sky.delays(dm_max).max())
    ntime = 32 * ((gulp + md + wmax) // 32 + 1)
    g = ntime // gulp
    return g, (g + 1) * gulp - ntime, ntime


def place(rng, sky: Sky, gulp: int, dm_max: float, wmax: int, dm: float, fwhm_ms: float) -> int:
    """A channel-0 arrival sample inside the first searched window's output
    span whose whole dispersed sweep has arrived by the end of that gulp."""
    g, ws, _ = first_window(sky, gulp, dm_max, wmax)
    pad = wmax + int(4 * fwhm_ms / (sky.tsamp * 1000.0)) + 8
    lo = ws + pad
    hi = min(ws + gulp - pad, (g + 1) * gulp - int(sky.delays(dm).max()) - pad)
    return int(rng.integers(lo, max(lo + 1, hi)))


def config_plain(seed: int = 1, nchan: int = 512, gulp: int = 16384, dm_max: float = 500.0):
    """Plain single-beam search: 512 ch over 375-468.75 MHz, tsamp
    1.048576 ms, gulp 16384; noise N(128, 20), 4 RFI channels (sd 80), three
    +60 broadband impulses of 5 samples, one flat-spectrum burst at DM 300,
    FWHM 2 ms, band-integrated S/N 20; DM 0-500 at tolerance 1.25 for a
    0.5 ms pulse; widths 1..32; 7 sigma."""
    rng = np.random.default_rng(seed)
    tsamp = 1.048576e-3
    df = -(F0 - FLO) / nchan
    rfi = tuple(int(c) for c in rng.choice(nchan, 4, replace=False))
    sky = Sky(nchan, tsamp, F0, df, seed, 128.0, 20.0, rfi, 80.0, 0.0, [], [])
    g, ws, _ = first_window(sky, gulp, dm_max, 64)
    sky.spikes = [Spike(int(ws + rng.integers(0, gulp)), 5, 60.0) for _ in range(3)]
    amp = snr_amp(20.0, 20.0, nchan, 2.0, tsamp)
    sky.bursts = [Burst(place(rng, sky, gulp, dm_max, 64, 300.0, 2.0), 300.0, 2.0, amp, 0.0)]
    params = dict(nchan=nchan, nbeam=1, gulp=gulp, tsamp=tsamp, plan_dt=tsamp, f0_mhz=F0, df_mhz=df,
                  dm_min=0.0, dm_max=dm_max, dm_tol=1.25, ti_us=500.0, width_min=1, width_max=64, snr=7.0)
    return params, sky


def config_full(seed: int = 2, nchan: int = 2048, gulp: int = 65536, dm_max: float = 2000.0):
    """Full single beam: 2048 ch over 375-468.75 MHz, tsamp 0.524288 ms,
    gulp 65536; N(128, 16) with a +-30% bandpass slope, 2% RFI channels
    (sd x4), 10 broadband spikes, 8 bursts with DM U[100,1800], FWHM
    logU[0.5,10] ms, S/N 8-50, spectral index -2..2; DM 0-2000 at tolerance
    1.25; widths 1..256."""
    rng = np.random.default_rng(seed)
    tsamp = 0.524288e-3
    df = -(F0 - FLO) / nchan
    rfi = tuple(int(c) for c in rng.choice(nchan, max(1, nchan // 50), replace=False))
    sky = Sky(nchan, tsamp, F0, df, seed, 128.0, 16.0, rfi, 64.0, float(rng.choice([-0.6, 0.6])), [], [])
    g, ws, _ = first_window(sky, gulp, dm_max, 512)
    sky.spikes = [Spike(int(ws + rng.integers(0, gulp)), int(rng.integers(1, 6)), 40.0) for _ in range(10)]
    for _ in range(8):
        dm = float(rng.uniform(100, min(1800.0, dm_max)))
        fwhm = float(np.exp(rng.uniform(np.log(0.5), np.log(10.0))))
        snr = float(rng.uniform(8, 50))
        sky.bursts.append(Burst(place(rng, sky, gulp, dm_max, 512, dm, fwhm), dm, fwhm,
                                snr_amp(snr, 16.0, nchan, fwhm, tsamp), float(rng.uniform(-2, 2))))
    params = dict(nchan=nchan, nbeam=1, gulp=gulp, tsamp=tsamp, plan_dt=tsamp, f0_mhz=F0, df_mhz=df,
                  dm_min=0.0, dm_max=dm_max, dm_tol=1.25, ti_us=40.0, width_min=1, width_max=512, snr=7.0)
    return params, sky


def multibeam_gulp(skies, g: int, n: int) -> np.ndarray:
    """u8 [nbeam][n][nchan] for gulp g of every beam's sky."""
    return np.stack([s.gulp(g, n) for s in skies])


def config_batched(nbeam: int = 256, seed: int = 3, nchan: int = 1024, gulp: int = 32768):
    """Batched multi-beam: nbeam beams of 1024 ch over 375-468.75 MHz, tsamp
    1.048576 ms, gulp 32768; per-beam killmasks flagging 0-10% of channels,
    DM ceilings uniform in 1000-2000, 0-3 bursts per beam as in the plain
    configuration (FWHM 2 ms, S/N 20, flat spectrum, DM below the ceiling);
    widths 1..32, 7 sigma.  Returns (params, ceilings, killmask, skies)."""
    rng = np.random.default_rng(seed)
    tsamp = 1.048576e-3
    df = -(F0 - FLO) / nchan
    ceilings = rng.uniform(1000.0, 2000.0, nbeam).astype(np.float32)
    frac = rng.uniform(0.0, 0.10, nbeam)
    kill = (rng.random((nbeam, nchan)) >= frac[:, None]).astype(np.int32)
    skies = []
    for b in range(nbeam):
        rfi = tuple(int(c) for c in rng.choice(nchan, 4, replace=False))
        sky = Sky(nchan, tsamp, F0, df, seed * 100000 + b, 128.0, 20.0, rfi, 80.0, 0.0, [], [])
        for _ in range(int(rng.integers(0, 4))):
            dm = float(rng.uniform(50.0, float(ceilings[b]) * 0.9))
            sky.bursts.append(Burst(place(rng, sky, gulp, float(ceilings[b]), 64, dm, 2.0), dm, 2.0,
                                    snr_amp(20.0, 20.0, nchan, 2.0, tsamp), 0.0))
        skies.append(sky)
    params = dict(nchan=nchan, nbeam=nbeam, gulp=gulp, tsamp=tsamp, plan_dt=tsamp, f0_mhz=F0, df_mhz=df,
                  dm_min=0.0, dm_max=float(ceilings.max()), dm_tol=1.25, ti_us=40.0, width_min=1, width_max=64,
                  snr=7.0)
    return params, ceilings, kill, skies


def config_stream(nbeam: int = 64, seconds: float = 600.0, seed: int = 4, nchan: int = 1024, gulp: int = 8192):
    """Streaming serving loop: nbeam beams of 1024 ch, tsamp 1.048576 ms, gulps
    of 8192 samples for `seconds` of sky.  RFI occupancy drifts between 0 and
    20% of the channels over the run; each beam gets one burst per 30 s on
    average (DM U[50, 2000], FWHM 2 ms, S/N 20).  Returns (params, ngulps,
    skies_at) where skies_at(g) gives every beam's sky model for gulp g (its
    RFI channels of that time)."""
    rng = np.random.default_rng(seed)
    tsamp = 1.048576e-3
    df = -(F0 - FLO) / nchan
    ngulps = int(math.ceil(seconds / (gulp * tsamp)))
    per_gulp = gulp * tsamp / 30.0
    skies = []
    for b in range(nbeam):
        sky = Sky(nchan, tsamp, F0, df, seed * 100000 + b, 128.0, 20.0, (), 80.0, 0.0, [], [])
        for g in range(ngulps):
            if rng.random() < per_gulp:
                dm = float(rng.uniform(50.0, 2000.0))
                sky.bursts.append(Burst(int(g * gulp + rng.integers(0, gulp)), dm, 2.0,
                                        snr_amp(20.0, 20.0, nchan, 2.0, tsamp), 0.0))
        skies.append(sky)
    order = rng.permutation(nchan)
    phase = rng.uniform(0, 2 * math.pi, nbeam)

    def skies_at(g: int):
        out = []
        for b, sky in enumerate(skies):
            occ = 0.10 + 0.10 * math.sin(2 * math.pi * g / max(1, ngulps) + phase[b])  # 0..20 %
            k = int(round(occ * nchan))
            out.append(dc.replace(sky, rfi_chans=tuple(int(c) for c in order[:k])))
        return out

    params = dict(nchan=nchan, nbeam=nbeam, gulp=gulp, tsamp=tsamp, plan_dt=tsamp, f0_mhz=F0, df_mhz=df,
                  dm_min=0.0, dm_max=2000.0, dm_tol=1.25, ti_us=40.0, width_min=1, width_max=64, snr=7.0)
    return params, ngulps, skies_at


def refine_truth(n: int, dm_grid: np.ndarray, nchan: int = 1024, nsamp: int = 2048, seed: int = 5,
                 tsamp: float = 1.048576e-3):
    """Candidate-refinement cutouts: n bursts with DM U[100,2000], FWHM
    U[0.5,20] ms, band-integrated S/N U[6,40], spectral index U[-3,3], near
    the cutout centre, in N(0,1) noise.  Each cutout is pre-dedispersed at
    its detection DM (the nearest trial of dm_grid) and the fit starts from
    the detection grid: that DM, the nearest boxcar width 2^k samples
    (k = 0..5), the detection sample, amplitude within +-30% of the truth,
    index 0.  Returns (theta_true [n,5], dm_ref [n], theta0 [n,5]) as f32,
    theta = (dm, t0 samples, width ms, amp, index)."""
    rng = np.random.default_rng(seed)
    df = -(F0 - FLO) / nchan
    fc = F0 - np.arange(nchan) * abs(df)
    tab = (4.148808e3 / tsamp * (1.0 / fc**2 - 1.0 / F0**2)).astype(np.float32).astype(np.float64)
    lnf = np.log(fc / F0)
    dm = rng.uniform(100.0, 2000.0, n)
    width = rng.uniform(0.5, 20.0, n)
    snr = rng.uniform(6.0, 40.0, n)
    idx = rng.uniform(-3.0, 3.0, n)
    dm_ref = dm_grid[np.abs(dm_grid[None, :] - dm[:, None]).argmin(axis=1)].astype(np.float32)
    sigma = width / (2.0 * math.sqrt(2.0 * math.log(2.0)) * tsamp * 1e3)
    s2 = np.exp(2.0 * idx[:, None] * lnf[None, :]).sum(axis=1)
    amp = snr / np.sqrt(s2 * sigma * math.sqrt(math.pi))
    t0 = nsamp / 2 + rng.uniform(-8.0, 8.0, n)
    resid = ((dm - dm_ref)[:, None] * tab[None, :]).mean(axis=1)
    t_det = np.round(t0 + resid)
    k = np.clip(np.round(np.log2(np.maximum(width / (tsamp * 1e3), 1.0))), 0, 5)
    w_det = 2.0 ** k * tsamp * 1e3
    truth = np.stack([dm, t0, width, amp, idx], axis=1).astype(np.float32)
    theta0 = np.stack([dm_ref, t_det, w_det, amp * rng.uniform(0.7, 1.3, n), np.zeros(n)], axis=1)
    return truth, dm_ref, theta0.astype(np.float32)


def refine_cutouts_device(truth: np.ndarray, dm_ref: np.ndarray, nchan: int, nsamp: int, out, seed: int = 6,
                          tsamp: float = 1.048576e-3, chunk: int = 32):
    """Fills the CUDA tensor out [n][nchan][nsamp] with model(truth) +
    N(0,1), evaluated with torch on the GPU in fp32 (the refinement model of
    include/hella_refine.h, pre-dedispersed at dm_ref)."""
    import torch

    df = -(F0 - FLO) / nchan
    fc = F0 - np.arange(nchan) * abs(df)
    tab32 = (4.148808e3 / tsamp * (1.0 / fc**2 - 1.0 / F0**2)).astype(np.float32)
    tab = torch.from_numpy(tab32).cuda()
    lnf = torch.from_numpy(np.log(fc / F0).astype(np.float32)).cuda()
    t = torch.arange(nsamp, device="cuda", dtype=torch.float32)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    c_w = 1.0 / (2.0 * math.sqrt(2.0 * math.log(2.0)) * tsamp * 1e3)
    th = torch.from_numpy(truth).cuda()
    dr = torch.from_numpy(dm_ref).cuda()
    for a in range(0, truth.shape[0], chunk):
        b = min(a + chunk, truth.shape[0])
        dm, t0, w, amp, idx = (th[a:b, k] for k in range(5))
        off = torch.floor(dr[a:b, None] * tab[None, :] + 0.5)
        mu = t0[:, None] + dm[:, None] * tab[None, :] - off
        sig = (w * c_w)[:, None, None]
        u = (t[None, None, :] - mu[:, :, None]) / sig
        m = (amp[:, None] * torch.exp(idx[:, None] * lnf[None, :]))[:, :, None] * torch.exp(-0.5 * u * u)
        out[a:b] = m + torch.randn(m.shape, generator=gen, device="cuda")
    return out
