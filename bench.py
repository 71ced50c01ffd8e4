#!/usr/bin/env python3
"""Real-time factor of the per-gulp FRB search on GB300.

Workload (the configuration the headline metric is quoted on): one beam of
uint8 filterbank, 2048 channels over 375-468.75 MHz, tsamp 0.524288 ms,
gulps of 65536 samples (34.36 s of sky) with max-delay overlap, DM 0-2000
at smearing tolerance 1.25 (2501 trials), smoothing widths 1..256, 7 sigma.
A step is one gulp through the whole path: flag + normalise + requantise,
dedisperse, smooth + standardise, find peaks, rewind.  Synthetic seeded
data (noise with bandpass slope, RFI channels, spikes, 8 dispersed bursts).

value: beam-seconds searched per wall second with the gulp already in HBM
(CUDA events on the search stream).  e2e: the same through the public C ABI
(hella_process_gulp) from pinned host memory, H2D of the gulp and D2H of
the candidates inside the timed region, with per-gulp p50/p99 latency.

--impl reference: the reference path's CPU implementation (the oracle
port; the reference itself has no CPU path and does not build here) on the
host cores, one whole searched gulp per step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "casm-hella_gb300"))

WORKLOAD = ("full single beam: 2048 ch 375-468.75 MHz, tsamp 0.524288 ms, gulp 65536, "
            "DM 0-2000 tol 1.25, widths 1-256, 7 sigma")
METRIC = "real-time factor (beam·s searched per s) at DM 0–2000; p99 gulp latency"
UNIT = "beam·s/s"
# dram__bytes_read.sum + dram__bytes_write.sum of one timed dedispersion launch of the full
# single beam, by tile shape (hella_tuning fields in order), from single-pass ncu captures of
# those two metrics on `bench.py --steps 3 --warmup 3 --no-cpu-baseline --no-batched` (one pass
# each, checked on the 512-channel case first).  A shape without a capture reports null.
DEDISP_TRAFFIC = {
    (0, 4, 8, 0, 8, 2): 8.664e9,  # 16-trial tiles, 8-channel stages, groups of 8, add mode 2: 7.99 + 0.673 GB
    # pair rows (add mode 5), 8 pairs a stage, groups of 8: k_pair_build 0.707 read + 5.78 written,
    # k_pair_sum 13.18 read + 0.654 written (profiles/k_pair_full_beam.md)
    (16, 4, 16, 0, 8, 5): 20.32e9,
    # rows of channel quads (add mode 6), 8 quads a stage, groups of 8: k_pair_build<4> 0.760 read +
    # 18.95 written, k_pair_sum 22.20 read + 0.657 written
    (16, 4, 16, 0, 8, 6): 42.57e9,
    # the same in groups of 4 (the bench's shape), rows kept as per-tile windows where those are
    # shorter than a tile, three staging buffers: 0.718 read + 14.88 written, 23.70 + 0.652
    (16, 4, 16, 0, 4, 6): 39.95e9,
}


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="full", choices=["full", "plain", "batched", "stream", "refine"],
                    help="full: the single-beam headline workload; batched: all beams of the "
                         "multi-beam configuration per step")
    ap.add_argument("--beams", type=int, default=256, help="beams of the batched workload")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the multi-beam leg that the full workload's line carries as `batched`")
    ap.add_argument("--batched-steps", type=int, default=8, help="timed gulps of that leg")
    ap.add_argument("--widths-per-pass", type=int, default=0,
                    help="smoothing widths whose planes the batched context holds at once (0: as many "
                         "as the free device memory allows); fewer hold less memory and re-read the "
                         "dedispersed planes once per extra pass")
    ap.add_argument("--seconds", type=float, default=600.0, help="sky seconds of the stream workload")
    ap.add_argument("--cutouts", type=int, default=4096, help="cutouts of the refine workload")
    ap.add_argument("--nchan", type=int, default=0,
                    help="channels of the full workload (0: 2048); smaller values give the small "
                         "cases that profiling captures use")
    ap.add_argument("--dm-max", type=float, default=0.0,
                    help="DM ceiling of the full workload (0: 2000); a small profiling case")
    ap.add_argument("--add-mode", type=int, default=6,
                    help="dedispersion add mode of the single-beam workloads (hella_tuning.add_mode; 6 / 5: rows "
                         "of channel quads / pairs, else the channel-by-channel kernel's pipe balance)")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks

class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


# ------------------------------------------------------------- workload

DATA_FULL = "synthetic (seeded noise, RFI, spikes, 8 dispersed bursts)"
DATA_PLAIN = "synthetic (seeded noise, 4 RFI channels, 3 broadband impulses, one DM-300 burst)"
PLAIN_WORKLOAD = ("plain single beam: 512 ch 375-468.75 MHz, tsamp 1.048576 ms, gulp 16384, DM 0-500 tol 1.25 "
                  "(0.5 ms pulse), widths 1-32, 7 sigma, one DM-300 burst")


def job_rate(dist, units: float, seconds: float, device: str = "cuda"):
    """Whole-job throughput of independent replicas: the units every rank
    processed over the slowest rank's time.  Returns (rate, slowest seconds).
    The ranks exchange no data; these two reductions are the only collectives."""
    if dist is None:
        return units / seconds, seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(t.item())


def workload(rank: int, ngulps: int = 3, which: str = "full", nchan: int = 0, dm_max: float = 0.0):
    import synth

    if which == "plain":
        params, sky = synth.config_plain(seed=1 + rank)
    elif nchan or dm_max:
        params, sky = synth.config_full(seed=2 + rank, nchan=nchan or 2048, dm_max=dm_max or 2000.0)
    else:
        params, sky = synth.config_full(seed=2 + rank)
    gulps = [sky.gulp(g, params["gulp"]) for g in range(ngulps)]
    return params, sky, gulps


def oracle_gulps(params, gulps, nsearch: int, nwarm: int = 0):
    """The oracle pipeline (the reference path restated on the CPU: flag,
    normalise, requantise, dedisperse every trial, smooth, standardise, find
    peaks, with the ring carried across gulps) on `nsearch` whole searched
    gulps, all host threads.  The ring is filled first and `nwarm` gulps are
    flagged, both untimed; `gulps` are reused in turn.  Returns (seconds per
    searched gulp, threads, description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.set_threads(0)
    pl = oracle.Pipeline.from_params(params, nbeam=1)
    gi = 0
    for _ in range(pl.min_gulp):
        pl.gulp_step(gulps[gi % len(gulps)][None])
        gi += 1
    for _ in range(nwarm):
        oracle.flag_beam(gulps[gi % len(gulps)])
    times = []
    for _ in range(nsearch):
        t0 = time.perf_counter()
        _, searched = pl.gulp_step(gulps[gi % len(gulps)][None])
        times.append(time.perf_counter() - t0)
        assert searched
        gi += 1
    pl.close()
    cores = os.cpu_count()
    desc = (f"oracle port on {cores} threads ({cpu_model()}): {nsearch} whole searched gulp(s) of "
            f"{params['nchan']} ch x {params['gulp']} samples, all {pl.ndms} DM trials, timed end to end "
            f"({np.mean(times):.1f} s each)")
    return times, cores, desc


def cpu_model() -> str:
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                return v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "model name" and v.strip():
                return v.strip()
    except OSError:
        pass
    import platform

    return platform.machine()


# ---------------------------------------------------------------- main

def main():
    a = args_()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if a.impl == "gb300" else "gloo")
    if a.impl == "reference":
        return run_reference(a, rank, world)

    torch.cuda.set_device(local)
    if a.workload == "batched":
        return main_batched(a, rank, world, local, dist)
    if a.workload == "stream":
        return main_stream(a, rank, world, local, dist)
    if a.workload == "refine":
        return main_refine(a, rank, world, local, dist)
    import hella_gb300 as hg

    hg.lib()
    if (a.nchan or a.dm_max) and a.workload != "full":
        raise SystemExit("--nchan and --dm-max apply to the full workload only")
    params, sky, gulps = workload(rank, which=a.workload, nchan=a.nchan, dm_max=a.dm_max)
    G, nch = params["gulp"], params["nchan"]
    gulp_s = G * params["tsamp"]
    s = hg.Search(hg.default_params(**params, device=local))
    info = s.info
    stream = torch.cuda.current_stream()
    s.set_stream(stream.cuda_stream)
    dev = [torch.from_numpy(g).cuda() for g in gulps]
    host = [torch.from_numpy(g).pin_memory() for g in gulps]

    ev = lambda: torch.cuda.Event(enable_timing=True)
    dd_ms, sm_ms, fl_ms = [], [], []

    def step(i, timed):
        e = [ev() for _ in range(4)] if timed else None
        s.clear_peaks()
        s.load_gulp(dev[i % len(dev)].data_ptr(), on_device=True)
        if timed:
            e[0].record(stream)
        s.fast_flagger()
        if timed:
            e[1].record(stream)
        s.dedisperse(0)
        if timed:
            e[2].record(stream)
        s.smooth(1)
        if timed:
            e[3].record(stream)
        s.find_peaks(0)
        s.rewind()
        return e

    # fill the ring, then warm up on searched gulps
    gi = 0
    for _ in range(info.min_gulp + a.warmup):
        step(gi, False)
        gi += 1
    torch.cuda.synchronize()
    # dedispersion: rows of channel quads (add mode 6: 16-trial tiles, 8 quads a stage, the deepest
    # staging that fits, DM tiles walked in groups of 4 per time tile), 9.8 ms on the full beam
    # (the autotuner's pick is within 1 %); pairs (add mode 5) 12.4 ms; the channel-by-channel
    # kernel's best shape (add mode 2, multiply-add odd lanes and addresses) 19.4 ms.  Shapes a DM
    # list or the memory cannot take fall back in that order, then to add mode 0.
    # The two row shapes are timed (3 runs each) and the faster kept: quads on the full beam, pairs
    # on the plain configuration's 16384-sample gulps (0.239 against 0.251 ms).
    rows = []
    for m in (6, 5):
        if m <= a.add_mode and a.add_mode >= 5:
            t = hg.HellaTuning(16, 4, 16, 0, 4 if m == 6 else 8, m)
            try:
                rows.append((s.time_dedisp(t, 3), m, t))
            except hg.HellaError:
                continue
    shapes = [t for _, _, t in sorted(rows, key=lambda r: (r[0], r[1]))]
    shapes += [hg.HellaTuning(0, 4, 8, 0, 8, a.add_mode if a.add_mode < 5 else 2), hg.HellaTuning(0, 4, 8, 0, 8, 0)]
    for shape in shapes:
        try:
            s.set_tuning(shape)
            s.time_dedisp(None, 1)
            break
        except hg.HellaError:
            continue

    # ---------------- device-resident timing
    clocks = Clocks(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = hg.kernel_launches()
    t0, t1 = ev(), ev()
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed steps' launches
    t0.record(stream)
    marks = []
    for _ in range(a.steps):
        marks.append(step(gi, True))
        gi += 1
    t1.record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    launches = hg.kernel_launches() - l0
    if dist:
        dist.barrier()
    ms = t0.elapsed_time(t1)
    for e in marks:
        fl_ms.append(e[0].elapsed_time(e[1]))
        dd_ms.append(e[1].elapsed_time(e[2]))
        sm_ms.append(e[2].elapsed_time(e[3]))
    value, slowest = job_rate(dist, a.steps * gulp_s, ms / 1e3)
    ms = slowest * 1e3
    ms_step = ms / a.steps

    # ---------------- end to end through the C ABI from pinned host memory
    lat = []
    ncand = []
    e2e_ev = [(ev(), ev()) for _ in range(a.steps)]
    for k in range(len(host)):  # untimed: each pinned buffer's first copy maps its pages for the copy engine
        s.process_gulp(host[(gi + k) % len(host)].data_ptr(), on_device=False)
    gi += len(host)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    w0 = time.perf_counter()
    for k in range(a.steps):
        q0 = time.perf_counter()
        e2e_ev[k][0].record(stream)
        cands, searched = s.process_gulp(host[gi % len(host)].data_ptr(), on_device=False)
        e2e_ev[k][1].record(stream)
        lat.append(time.perf_counter() - q0)
        ncand.append(len(cands))
        gi += 1
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - w0
    # the stream's own time for each call (upload, search, candidate copy): a host-side stall
    # shows as latency above it
    e2e_dev = [e0.elapsed_time(e1) for e0, e1 in e2e_ev]
    e2e, e2e_s = job_rate(dist, a.steps * gulp_s, e2e_s)

    # ---------------- end to end through the serving API: the same gulps through a one-beam
    # batched context with two gulps in flight (hella_batch_submit / hella_batch_poll), each
    # gulp's upload overlapping the search of the gulp before; same tile shape
    bt1 = hg.Batch(hg.default_params(**params, device=local), inflight=2)
    bt1.set_tuning(s.get_tuning())
    for k in range(info.min_gulp + 2):  # fill the ring, then warm up on searched gulps
        bt1.submit(host[gi % len(host)].data_ptr())
        bt1.poll()
        gi += 1
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    pend, pipe_dev, pipe_n = 0, [], []
    w1 = time.perf_counter()
    for k in range(a.steps):
        bt1.submit(host[gi % len(host)].data_ptr())
        gi += 1
        pend += 1
        if pend == 2:
            got1, _, _, _, d1 = bt1.poll()
            pipe_dev.append(d1), pipe_n.append(len(got1))
            pend -= 1
    while pend:
        got1, _, _, _, d1 = bt1.poll()
        pipe_dev.append(d1), pipe_n.append(len(got1))
        pend -= 1
    pipe_s = time.perf_counter() - w1
    e2e_pipe, _ = job_rate(dist, a.steps * gulp_s, pipe_s)
    bt1.close()

    clk = clocks.stop()

    # ---------------- rooflines
    nact = nch
    adds = float(info.ndms) * nact * info.ntime_dd
    dd_t = float(np.mean(dd_ms)) / 1e3
    peak_int = 2 * hg.int_add_peak(local) / 1e12  # two u8 sums per 32-bit add (16-bit SWAR lanes)
    peak_smem = hg.smem_read_peak(local) / 1e12
    achieved = adds / dd_t / 1e12
    pairs = s.get_tuning().add_mode >= 5
    work = f"{info.ndms} trials x {nact} ch x {info.ntime_dd} samples"
    traffic = (DEDISP_TRAFFIC.get(tuple(s.get_tuning().as_dict().values()))
               if a.workload == "full" and not (a.nchan or a.dm_max) else None)
    mode = s.get_tuning().add_mode
    kernel = (f"k_pair_build + k_pair_sum (add mode {mode}: rows of channel {'quads' if mode == 6 else 'pairs'}, "
              "timed together)") if pairs else "k_dedisp"
    # one yardstick for every form of the dedispersion: channel-sample adds against the measured
    # SWAR integer-add ceiling (two u8 sums per 32-bit add), the bound of the channel-by-channel
    # kernel; the row kernels' own bound, shared-memory reads, is reported beside it
    roof = {"bound": "int32", "achieved": round(achieved, 3), "peak": round(peak_int, 3), "unit": "Tadd/s",
            "frac": round(achieved / peak_int, 4),
            "peak_source": "measured: register-only 32-bit add chains on all SMs (hella_int_add_peak) x2 lanes",
            "ms_per_launch": round(dd_t * 1e3, 3), "kernel": kernel, "work_per_launch": work, "traffic": traffic,
            "traffic_unit": "bytes per launch (ncu" + (", both kernels)" if pairs else ")")}
    # shared-memory bytes read per channel-sample: 1 for pairs and the channel-by-channel kernel, 1/2 for quads
    smem_b = 0.5 if mode == 6 else 1.0
    smem_roof = {"bound": "smem", "achieved": round(achieved * smem_b, 3), "peak": round(peak_smem, 3),
                 "unit": "TB/s", "frac": round(achieved * smem_b / peak_smem, 4),
                 "peak_source": "measured: conflict-free 16-byte shared-memory loads on all SMs "
                                "(hella_smem_read_peak)",
                 "note": f"{smem_b:g} byte read per channel-sample over the time of the whole dedispersion"
                         + (" (row build included)" if pairs else ""),
                 "ms_per_launch": round(dd_t * 1e3, 3)}
    hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs") if (
        ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    sm_t = float(np.mean(sm_ms)) / 1e3
    plane = 4.0 * info.ndms * info.ntime_dd
    boxes = 4.0 * info.nboxcar * (info.ndms - 2) * info.ntime_out
    smooth_bytes = 3 * plane + boxes * 3 + 4.0 * (info.ndms - 2) * info.ntime_out * 2
    fl_t = float(np.mean(fl_ms)) / 1e3
    flag_bytes = 10.0 * nch * G
    extra = {
        "smooth": {"bound": "hbm", "achieved": round(smooth_bytes / sm_t / 1e9, 1), "peak": hbm, "unit": "GB/s",
                   "frac": round(smooth_bytes / sm_t / 1e9 / hbm, 4), "ms_per_launch": round(sm_t * 1e3, 3),
                   "note": "FIR + per-width statistics; bytes = dd plane read x3 + planes write/read; the FIR "
                           "itself is FP32-FMA issue bound (profiles/)"},
        "flagger": {"bound": "hbm", "achieved": round(flag_bytes / fl_t / 1e9, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(flag_bytes / fl_t / 1e9 / hbm, 4), "ms_per_launch": round(fl_t * 1e3, 3),
                    "note": "9 u8 passes + 1 u8 write per sample"},
    }
    extra["dedisp_smem"] = smem_roof
    if roof["traffic"]:
        # the dominant kernel against HBM: its measured DRAM traffic over the launch time
        gbs = roof["traffic"] / dd_t / 1e9
        extra["dedisp_hbm"] = {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s",
                               "frac": round(gbs / hbm, 4), "ms_per_launch": round(dd_t * 1e3, 3),
                               "note": "the dedispersion's ncu DRAM bytes per launch over its time"}

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8",
        "data": DATA_PLAIN if a.workload == "plain" else DATA_FULL,
        "config": {"workload": PLAIN_WORKLOAD if a.workload == "plain" else
                   WORKLOAD.replace("2048 ch", f"{nch} ch").replace("DM 0-2000", f"DM 0-{params['dm_max']:g}"),
                   "nchan": nch, "gulp": G,
                   "tsamp": params["tsamp"],
                   "ndms": info.ndms, "max_delay": info.max_delay, "ntime": info.ntime,
                   "widths": info.nboxcar, "beams_per_gpu": 1, "parallelism": f"replicas{world}",
                   "tuning": s.get_tuning().as_dict(),
                   "l2": (f"inputs {'larger' if info.ndms * info.ntime_dd * 4 > 129e6 else 'smaller'} than L2: "
                          f"{G * nch / 1e6:.0f} MB gulp, {nch * info.ntime * 5 / 1e9:.2f} GB ring, "
                          f"{info.ndms * info.ntime_dd * 4 / 1e9:.2f} GB plane, "
                          f"{info.nboxcar * (info.ndms - 2) * G * 4 / 1e9:.2f} GB smoothed planes")},
        # value: the serving API (two gulps in flight, uploads overlapped); latencies: each gulp's
        # synchronous call through the stage API (hella_process_gulp), whose rate is `sync_value`
        "e2e": {"value": round(e2e_pipe, 2), "unit": UNIT, "h2d_bytes_per_step": G * nch,
                "d2h_bytes_per_step": int(4 + 20 * np.mean(pipe_n)),
                "api": "hella_batch_submit / hella_batch_poll, one beam, two gulps in flight",
                "period_ms": round(pipe_s / a.steps * 1e3, 3),
                "device_ms_p50": round(float(np.percentile(pipe_dev, 50)), 3),
                "sync_value": round(e2e, 2), "sync_api": "hella_process_gulp (pinned host gulp, synchronous)",
                "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                "max_ms": round(1e3 * max(lat), 2), "gulp_ms": round(gulp_s * 1e3, 1),
                "stream_ms_p50": round(float(np.percentile(e2e_dev, 50)), 2),
                "stream_ms_p99": round(float(np.percentile(e2e_dev, 99)), 2),
                "stream_ms_max": round(float(max(e2e_dev)), 2)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "rooflines_other": extra,
        "clocks": clk,
        "candidates_per_gulp": float(np.mean(ncand)),
    }
    s.close()
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        times, cores, desc = oracle_gulps(params, gulps, 1)
        line["cpu_baseline"] = {"value": round(gulp_s / times[0], 4), "unit": UNIT, "cores": cores,
                                "kind": "port", "sample": desc}
    if a.workload == "full" and not (a.nchan or a.dm_max) and not a.no_batched:
        # the multi-beam configuration under the same clock: 256 beams x 1024 ch, one graph per gulp
        del dev, host
        torch.cuda.empty_cache()
        bl = batched_leg(a, rank, world, local, dist, a.batched_steps, min(a.warmup, 3),
                         cpu=not a.no_cpu_baseline)
        line["batched"] = {k: bl[k] for k in ("value", "unit", "ms_per_step", "steps", "warmup", "config", "e2e",
                                              "gpu_launches", "roofline", "clocks", "candidates_per_gulp")
                           if k in bl}
        if "cpu_baseline" in bl:
            line["batched"]["cpu_baseline"] = bl["cpu_baseline"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


BATCH_WORKLOAD = ("batched multi-beam: {nb} beams x 1024 ch 375-468.75 MHz, tsamp 1.048576 ms, gulp 32768, "
                  "DM ceilings U[1000,2000] tol 1.25, killmasks 0-10%, widths 1-32, 7 sigma, one CUDA graph per gulp")


def batched_sample_params(params, ceiling):
    p = dict(params)
    p["dm_max"] = float(ceiling)
    return p


def main_batched(a, rank, world, local, dist):
    """All beams of the multi-beam configuration per step (hella_batch_*)."""
    line = batched_leg(a, rank, world, local, dist, a.steps, a.warmup, cpu=not a.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def batched_leg(a, rank, world, local, dist, steps: int, warmup: int, cpu: bool = True) -> dict:
    """Times `steps` gulps of every beam of the multi-beam configuration
    (one CUDA graph per gulp) device-resident, then end to end from pinned
    host memory with two gulps in flight; returns the JSON line's fields."""
    import torch
    import hella_gb300 as hg
    import synth

    params, ceilings, kill, skies = synth.config_batched(nbeam=a.beams, seed=3 + rank)
    NB, G, nch = params["nbeam"], params["gulp"], params["nchan"]
    gulp_s = G * params["tsamp"]
    ngen = 2
    dev = []
    for g in range(ngen):
        t = torch.empty((NB, G, nch), dtype=torch.uint8, device="cuda")
        for b in range(NB):
            synth.gulp_device(skies[b], g, G, out=t[b])
        dev.append(t)
    host = []
    for t in dev:
        h = torch.empty(t.shape, dtype=torch.uint8, pin_memory=True)
        h.copy_(t)
        host.append(h)
    torch.cuda.synchronize()
    t_c = time.perf_counter()
    bt = hg.Batch(hg.default_params(**params, device=local, autotune=1), dm_max=ceilings, killmask=kill,
                  inflight=2, widths_per_pass=a.widths_per_pass)
    create_s = time.perf_counter() - t_c
    infos = [bt.info(b) for b in range(NB)]
    tune = bt.get_tuning().as_dict()

    gi = 0
    for _ in range(max(i.min_gulp for i in infos) + warmup):
        bt.process_gulp(dev[gi % ngen].data_ptr(), on_device=True)
        gi += 1

    # ---------------- device-resident: the graph of one gulp, CUDA events
    clocks = Clocks(local)
    clocks.start()
    if dist:
        dist.barrier()
    dev_ms, ncand = [], []
    for _ in range(steps):
        got, counts, _ = bt.process_gulp(dev[gi % ngen].data_ptr(), on_device=True)
        dev_ms.append(bt.last_gulp_ms())
        ncand.append(len(got))
        gi += 1
    value, slowest = job_rate(dist, steps * NB * gulp_s, float(np.sum(dev_ms)) / 1e3)
    ms = slowest * 1e3

    # ---------------- end to end from pinned host memory: two gulps in flight, the upload of
    # gulp k+1 overlapping the search of gulp k (hella_batch_submit / hella_batch_poll)
    lat, e2e_dev, polled = [], [], []
    # untimed warm-up of both lanes (each lane's graph is built on its first use)
    for _ in range(2):
        bt.submit(host[gi % ngen].data_ptr())
        gi += 1
    for _ in range(2):
        bt.poll()
    if dist:
        dist.barrier()
    w0 = time.perf_counter()
    bt.submit(host[gi % ngen].data_ptr())
    first_submit_ms = 1e3 * (time.perf_counter() - w0)
    gi += 1
    for k in range(steps):
        if k + 1 < steps:
            bt.submit(host[gi % ngen].data_ptr())
            gi += 1
        got, counts, _, l_ms, d_ms = bt.poll()
        polled.append(time.perf_counter())
        lat.append(l_ms / 1e3)
        e2e_dev.append(d_ms)
    e2e_s = time.perf_counter() - w0
    # gulp to gulp once the pipeline is full (the first gulp's upload is not overlapped)
    steady = np.diff(polled) * 1e3 if len(polled) > 1 else np.asarray([e2e_s * 1e3])
    e2e, e2e_s = job_rate(dist, steps * NB * gulp_s, e2e_s)
    clk = clocks.stop()

    # ---------------- dedispersion roofline: the all-beam launch alone
    dd_ms = bt.time_dedisp(reps=3)
    adds = float(sum(i.ndms * int(kill[b].sum()) * i.ntime_dd for b, i in enumerate(infos)))
    peak = 2 * hg.int_add_peak(local) / 1e12
    achieved = adds / (dd_ms / 1e3) / 1e12
    dd_kernel = ("k_pair_build + k_pair_sum (add mode {m}: rows of channel {g}, beams in chunks of up to four "
                 "per launch pair, timed together)".format(m=tune["add_mode"],
                                                           g="quads" if tune["add_mode"] == 6 else "pairs")
                 if tune["add_mode"] >= 5 else "k_dedisp (all beams, one launch)")
    roof = {"bound": "int32", "achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "Tadd/s",
            "frac": round(achieved / peak, 4), "traffic": None, "kernel": dd_kernel,
            "work_per_launch": f"sum over {NB} beams of trials x unkilled channels x {infos[0].ntime_dd} samples",
            "peak_source": "measured: register-only 32-bit add chains on all SMs (hella_int_add_peak) x2 lanes",
            "ms_per_launch": round(dd_ms, 3)}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": round(ms / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded noise, RFI channels, 0-3 dispersed bursts per beam; drawn on the GPU)",
        "config": {"workload": BATCH_WORKLOAD.format(nb=NB), "beams": NB, "nchan": nch, "gulp": G,
                   "tsamp": params["tsamp"], "ndms_min": min(i.ndms for i in infos),
                   "ndms_max": max(i.ndms for i in infos), "ntime_max": max(i.ntime for i in infos),
                   "widths": infos[0].nboxcar, "tuning": tune, "create_s": round(create_s, 2),
                   "device_gb": round(infos[0].device_bytes / 1e9, 1), "widths_per_pass": a.widths_per_pass or "all",
                   "parallelism": f"replicas{world}",
                   "real_time_x": round(value / NB, 2),
                   "l2": f"inputs larger than L2: {NB * G * nch / 1e9:.1f} GB gulp per step"},
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": NB * G * nch,
                "d2h_bytes_per_step": int(4 * NB + 20 * np.mean(ncand)), "inflight": 2,
                "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                "max_ms": round(1e3 * max(lat), 2), "gulp_ms": round(gulp_s * 1e3, 1),
                "device_ms_p50": round(float(np.percentile(e2e_dev, 50)), 2),
                "period_ms": round(1e3 * e2e_s / steps, 2),
                "first_gulp_ms": round(1e3 * (polled[0] - w0), 2),
                "first_gulp_device_ms": round(float(e2e_dev[0]), 2),
                "first_submit_ms": round(first_submit_ms, 2),
                "latency_ms_each": [round(1e3 * x, 1) for x in lat],
                "device_ms_each": [round(float(x), 1) for x in e2e_dev],
                "steady_period_ms_p50": round(float(np.percentile(steady, 50)), 2)},
        "gpu_launches": int(steps * 2 * bt.graph_kernels()),
        "roofline": roof,
        "clocks": clk,
        "candidates_per_gulp": float(np.mean(ncand)),
    }
    if rank == 0 and world == 1 and cpu:
        gl = [skies[0].gulp(g, G) for g in range(infos[0].min_gulp + 1)]
        p0 = batched_sample_params(params, ceilings[0])
        p0["nbeam"] = 1
        times, cores, desc = oracle_gulps(p0, gl, 1)
        line["cpu_baseline"] = {"value": round(gulp_s / times[0], 4), "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "beam 0 of the batch (its own DM ceiling), one beam per wall second: "
                                          + desc + "; beams are independent, so the batch's CPU time scales "
                                                   f"with the {NB} beams"}
    bt.close()
    return line


STREAM_WORKLOAD = ("streaming serving loop: 64 beam requests x 1024 ch, tsamp 1.048576 ms, gulps of 8192 "
                   "samples for {sec:.0f} s of sky, DM 0-2000, widths 1-32, slots admitted by an HBM budget, "
                   "beams joining and leaving, RFI occupancy drifting 0-20%, two gulps in flight")


def main_stream(a, rank, world, local, dist):
    """The serving loop of the streaming configuration (submit/poll): the
    whole schedule of joins and leaves run twice, gulps back to back
    (throughput) and gulps released at a fixed arrival period (latency from
    a gulp's arrival to its candidates on the host)."""
    import torch
    import hella_gb300 as hg
    import synth

    params, ngulps, skies_at = synth.config_stream(seconds=a.seconds, seed=4 + rank)
    NB, G, nch = params["nbeam"], params["gulp"], params["nchan"]
    gulp_s = G * params["tsamp"]
    kw = dict(dynamic=True, inflight=2)
    # the HBM budget: 3/4 of what all 64 requests need with every smoothing width's planes held
    need = hg.batch_bytes(hg.default_params(**params), **kw)
    budget = int(0.75 * need)
    # admission: the most slots whose state fits the budget with one width's planes held at a
    # time (the smoothing then runs one width per pass; each pass re-reads the dedispersed plane)
    fit = lambda n, w: hg.batch_bytes(hg.default_params(**dict(params, nbeam=n, hbm_budget=budget)),
                                      widths_per_pass=w, **kw)
    slots = NB
    while slots > 1 and fit(slots, 1) > budget:
        slots -= 1
    per_width = fit(slots, 2) - fit(slots, 1)
    nbox = len([w for w in range(16) if params["width_min"] << w < params["width_max"]])
    wpp = int(min(nbox, (budget - (fit(slots, 1) - per_width)) // per_width))
    # dedispersion through rows of channel pairs (add mode 5: on these 8192-sample gulps pairs and
    # quads both take 33.6 ms for all 64 slots against 41.3 ms channel by channel, and pair rows
    # are the smaller) when their rows -- up to four slots' worth -- and tables fit in the same
    # budget beside the slots, paid for with smoothing widths per pass (each extra pass re-reads
    # the dedispersed planes); sized from the plan's own tables
    ntt = -(-(G + params["width_max"]) // 1024)
    pl = hg.Plan(nch, params["plan_dt"], params["f0_mhz"], params["df_mhz"])
    pl.generate_dm_list(params["dm_min"], params["dm_max"], params["ti_us"], params["dm_tol"])
    tab = pl.pair_tables(0, pl.dm_count, 2, 8, ntt)
    pl.close()
    rows_bytes = (4 * tab["words"] * 4 + tab["rec"].nbytes + 64 * tab["nrows"] + slots * nch * 2
                  + (16 << 20))
    wpp_rows = int(min(nbox, (budget - rows_bytes - (fit(slots, 1) - per_width)) // per_width))
    use_rows = wpp_rows >= 1
    if use_rows:
        wpp = wpp_rows
    shape = hg.HellaTuning(16, 4, 16, 0, 4, 5) if use_rows else hg.HellaTuning(0, 4, 8, 0, 8, 2)
    rng = np.random.default_rng(7 + rank)
    # requests: 48 beams from the start, 16 more at 25% of the run; 12 leave at 50%
    join_at = {b: 0 if b < 48 else ngulps // 4 for b in range(NB)}
    leave_at = {int(b): ngulps // 2 for b in rng.choice(48, 12, replace=False)}
    kills = (rng.random((NB, nch)) >= rng.uniform(0, 0.1, (NB, 1))).astype(np.int32)

    # all gulps of the run, drawn on the GPU into pinned host memory before timing
    t_gen = time.perf_counter()
    host = torch.empty((ngulps, NB, G, nch), dtype=torch.uint8, pin_memory=True)
    buf = torch.empty((NB, G, nch), dtype=torch.uint8, device="cuda")
    for g in range(ngulps):
        sk = skies_at(g)
        for b in range(NB):
            synth.gulp_device(sk[b], g, G, out=buf[b])
        host[g].copy_(buf)
    del buf
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t_gen
    lanes = [torch.empty((slots, G, nch), dtype=torch.uint8, pin_memory=True) for _ in range(2)]

    def run(period_s: float):
        """The schedule once; period_s = 0: back to back with two gulps in
        flight, else gulp g arrives at g * period_s and is polled at once."""
        bt = hg.Batch(hg.default_params(**dict(params, nbeam=slots, device=local, hbm_budget=budget)),
                      member=np.zeros(slots, np.int32), widths_per_pass=wpp, **kw)
        bt.set_tuning(shape)
        slot_of, free, waiting = {}, list(range(slots)), []
        st = dict(admitted=0, waited=0, searched=0, lat=[], dev=[], ncand=[], arrival=[])
        pending = []

        def poll():
            got, counts, searched, l_ms, d_ms = bt.poll()
            arrived = pending.pop(0)
            st["arrival"].append((time.perf_counter() - arrived) * 1e3)
            st["lat"].append(l_ms), st["dev"].append(d_ms), st["ncand"].append(len(got))
            st["searched"] += int(searched.sum())

        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for g in range(ngulps):
            arrive = t0 + g * period_s
            if period_s:
                while time.perf_counter() < arrive:
                    time.sleep(min(0.002, max(0.0, arrive - time.perf_counter())))
            # membership changes need an idle batch: drain, then admit / release
            changes = [b for b, t in leave_at.items() if t == g and b in slot_of]
            arrivals = [b for b, t in join_at.items() if t == g]
            if changes or arrivals or (waiting and free):
                while pending:
                    poll()
                for b in changes:
                    sl = slot_of.pop(b)
                    bt.set_beam(sl, False)
                    free.append(sl)
                for b in arrivals:
                    waiting.append(b)
                    if not free:
                        st["waited"] += 1
                while waiting and free:
                    b, sl = waiting.pop(0), free.pop(0)
                    bt.set_beam(sl, True, params["dm_max"], kills[b])
                    slot_of[b] = sl
                    st["admitted"] += 1
            lane = lanes[g % 2]
            for b, sl in slot_of.items():
                lane[sl].copy_(host[g, b])
            bt.submit(lane.data_ptr())
            pending.append(arrive if period_s else time.perf_counter())
            if period_s or len(pending) == 2:
                poll()
        while pending:
            poll()
        st["wall"] = time.perf_counter() - t0
        st["kernels"] = int(ngulps * bt.graph_kernels())
        bt.close()
        return st

    clocks = Clocks(local)
    clocks.start()
    fast = run(0.0)
    period = max(0.05, 2.5 * float(np.percentile(fast["dev"], 99)) / 1e3)
    paced = run(period)
    clk = clocks.stop()
    beam_gulps = fast["searched"]
    value, _ = job_rate(dist, beam_gulps * gulp_s, float(np.sum(fast["dev"])) / 1e3)
    e2e, _ = job_rate(dist, beam_gulps * gulp_s, fast["wall"])
    arr = np.asarray(paced["arrival"])
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": ngulps,
        "warmup": 0, "ms_per_step": round(float(np.mean(fast["dev"])), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded noise, drifting RFI, bursts 1 per beam per 30 s; drawn on the GPU)",
        "config": {"workload": STREAM_WORKLOAD.format(sec=a.seconds), "beam_requests": NB,
                   "slots_in_budget": slots, "hbm_budget_gb": round(budget / 1e9, 2),
                   "widths_per_pass": wpp, "tuning": shape.as_dict(),
                   "rows_gb": round(rows_bytes / 1e9, 2) if use_rows else 0.0,
                   "admitted": fast["admitted"], "waited_for_a_slot": fast["waited"],
                   "gulps": ngulps, "searched_beam_gulps": beam_gulps,
                   "cadence": (f"value and e2e.value: gulps back to back, two in flight; e2e latencies: gulps "
                               f"released every {period * 1e3:.0f} ms (the 8.6 s real-time period compressed), "
                               f"arrival to candidates on the host"),
                   "gen_s": round(gen_s, 1), "parallelism": f"replicas{world}"},
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": slots * G * nch,
                "d2h_bytes_per_step": int(4 * slots + 20 * np.mean(fast["ncand"])),
                "p50_ms": round(float(np.percentile(arr, 50)), 2), "p99_ms": round(float(np.percentile(arr, 99)), 2),
                "max_ms": round(float(arr.max()), 2), "period_ms": round(period * 1e3, 1),
                "gulp_ms": round(gulp_s * 1e3, 1),
                "back_to_back_p50_ms": round(float(np.percentile(fast["arrival"], 50)), 2),
                "back_to_back_p99_ms": round(float(np.percentile(fast["arrival"], 99)), 2)},
        "gpu_launches": fast["kernels"],
        "clocks": clk,
        "candidates_per_gulp": float(np.mean(fast["ncand"])),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main_refine(a, rank, world, local, dist):
    """Differentiable refinement of the candidate cutouts: 50 Adam steps."""
    import torch
    import hella_gb300 as hg
    import synth

    n, nch, ns, ts = a.cutouts, 1024, 2048, 1.048576e-3
    df = -(synth.F0 - synth.FLO) / nch
    plan = hg.Plan(nch, ts, synth.F0, df)
    plan.generate_dm_list(0.0, 2000.0, 40.0, 1.25)
    truth, dm_ref, theta0 = synth.refine_truth(n, plan.dm_list(), nchan=nch, nsamp=ns, seed=5 + rank)
    cut = torch.empty((n, nch, ns), dtype=torch.float32, device="cuda")
    synth.refine_cutouts_device(truth, dm_ref, nch, ns, cut, seed=6 + rank)
    stream = torch.cuda.current_stream()
    r = hg.Refine(n, nch, ns, ts, synth.F0, df, device=local, stream=stream.cuda_stream)
    ddm = torch.from_numpy(dm_ref).cuda()
    lr = [0.5, 0.2, 0.05, 0.05, 0.05]
    steps = 50
    chi0 = torch.empty(n, device="cuda")
    r.forward(cut, ddm, torch.from_numpy(theta0).cuda(), chi0)
    for _ in range(a.warmup):                       # warm-up fits from the same start
        th = torch.from_numpy(theta0).cuda()
        r.fit(cut, ddm, th, 2, lr)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    theta = torch.from_numpy(theta0).cuda()
    chi = torch.empty(n, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    r.fit(cut, ddm, theta, steps, lr, chi)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # one fused pass alone, for the roofline
    g = torch.empty((n, 5), device="cuda")
    ones = torch.ones(n, device="cuda")
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(5):
        r.adjoint(cut, ddm, theta, ones, g)
    p1.record(stream)
    torch.cuda.synchronize()
    pass_ms = p0.elapsed_time(p1) / 5
    clk = clocks.stop()
    # end to end: cutouts from pinned host memory, fit, parameters back
    host = torch.empty(cut.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(cut)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    dcut = torch.empty_like(cut)
    dcut.copy_(host, non_blocking=True)
    th2 = torch.from_numpy(theta0).cuda()
    r.fit(dcut, ddm, th2, steps, lr)
    out = th2.cpu()
    e2e_s = time.perf_counter() - w0
    fit = theta.cpu().numpy()
    rate, _ = job_rate(dist, n, ms / 1e3)
    rate_e2e, _ = job_rate(dist, n, e2e_s)
    bytes_pass = float(n) * nch * ns * 4
    hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs") if (
        ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    ach = bytes_pass / (pass_ms / 1e3) / 1e9
    derr0 = np.abs(theta0[:, 0] - truth[:, 0])
    derr1 = np.abs(fit[:, 0] - truth[:, 0])
    line = {
        "metric": "candidate cutouts refined per second (50 Adam steps each)",
        "value": round(rate, 1), "unit": "cutouts/s", "n_gpus": world, "steps": steps,
        "warmup": a.warmup, "ms_per_step": round(ms / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (dispersed Gaussian bursts in N(0,1) noise, drawn on the GPU)",
        "config": {"workload": f"differentiable refinement: {n} cutouts of 1024 ch x 2048 samples, "
                               f"tsamp 1.048576 ms, DM 100-2000, width 0.5-20 ms, S/N 6-40, index -3..3, "
                               f"{steps} Adam steps from the detection grid",
                   "cutout_gb": round(bytes_pass / 1e9, 1),
                   "dm_abs_err_median": [round(float(np.median(derr0)), 3), round(float(np.median(derr1)), 3)],
                   "chi2_ratio_median": round(float(np.median((chi.cpu() / chi0.cpu()).numpy())), 4)},
        "e2e": {"value": round(rate_e2e, 1), "unit": "cutouts/s", "h2d_bytes_per_step": int(bytes_pass),
                "d2h_bytes_per_step": int(out.numel() * 4)},
        "gpu_launches": 2 * steps,
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(ach / hbm, 4), "traffic": None, "kernel": "k_refine<true>",
                     "work_per_launch": f"{n} x 1024 x 2048 fp32 read once", "ms_per_launch": round(pass_ms, 3)},
        "clocks": clk,
    }
    r.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_reference(a, rank, world):
    """The reference path's CPU implementation on the host cores: each step
    one whole searched gulp of the workload through the oracle pipeline (no
    extrapolation); the warm-up fills the ring and flags `warmup` gulps."""
    if rank != 0:
        return
    which = a.workload if a.workload in ("full", "plain") else "full"
    params, sky, gulps = workload(0, ngulps=3, which=which)
    gulp_s = params["gulp"] * params["tsamp"]
    times, cores, desc = oracle_gulps(params, gulps, a.steps, nwarm=a.warmup)
    per = float(np.mean(times))
    v = gulp_s / per
    line = {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(per * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": DATA_PLAIN if which == "plain" else DATA_FULL,
            "config": {"workload": PLAIN_WORKLOAD if which == "plain" else WORKLOAD}, "impl": "reference",
            "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
