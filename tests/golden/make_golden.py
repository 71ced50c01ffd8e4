"""Generate tests/golden/reference_fixtures.json from the reference's own
code (not part of the test run).

Builds the reference's flagger, statistics, median filter, smoothing and
peak-finding sources for the CPU under oracle/ref (the CUDA kernels run on
an emulator; see oracle/ref/emu_cuda.h), runs them on the seeded cases of
cases.py and records their outputs.  Needs the reference tree (the first argument, or $HELLA_REF); the tests only
read the JSON it writes.

    python tests/golden/make_golden.py <reference tree>
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle" / "ref"))
sys.path.insert(0, str(HERE))
import build_ref  # noqa: E402
import cases  # noqa: E402

VP = C.c_void_p


def main():
    lib = build_ref.build(build_ref.reference_tree(sys.argv), nchan=cases.NCHAN, verbose=True)
    R = C.CDLL(str(lib))
    R.ref_flag.argtypes = [VP, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, VP, VP, VP, VP, VP, VP]
    R.ref_stddev_f32.restype = C.c_float
    R.ref_stddev_f32.argtypes = [VP, C.c_int, C.c_int, C.c_int, VP]
    R.ref_stddev_f16.restype = C.c_float
    R.ref_stddev_f16.argtypes = [VP, C.c_int, C.c_int, C.c_int, VP]
    R.ref_median_filter.restype = C.c_float
    R.ref_median_filter.argtypes = [VP, VP, C.c_int, C.c_int]
    R.ref_smooth.argtypes = [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, VP, VP, C.c_int]
    R.ref_find_peaks.argtypes = [VP, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, VP, VP, VP, VP]
    assert R.ref_nchan() == cases.NCHAN
    out = {"generator": "tests/golden/make_golden.py", "nchan": cases.NCHAN, "flag": [], "stddev_f32": [],
           "stddev_f16": [], "median": [], "smooth": []}

    for c in cases.FLAG_CASES:
        x = cases.flag_input(c)
        w = c["w"]
        sc = c["scrunch"]
        t = np.array([s[0] for s in sc] or [0], np.int32)
        f = np.array([s[1] for s in sc] or [0], np.int32)
        th = np.array([s[2] for s in sc] or [0], np.float32)
        o = np.zeros((w, cases.NCHAN), np.uint8)
        ts = np.zeros(w, np.float32)
        fs = np.zeros(cases.NCHAN, np.float32)
        R.ref_flag(x.ctypes.data, w, -0.05, 0.15, c.get("flag1", -1), c.get("flag2", -1), len(sc), t.ctypes.data,
                   f.ctypes.data, th.ctypes.data, o.ctypes.data, ts.ctypes.data, fs.ctypes.data)
        out["flag"].append(dict(name=c["name"], out_sha=cases.sha(o), ts_sha=cases.sha(ts), ts_head=cases.bits(ts[:16]),
                                flagspec=cases.bits(fs), out_mean=float(o.mean())))

    for c in cases.STAT_CASES:
        x = cases.stat_input_f32(c)
        m = np.zeros(1, np.float32)
        s = R.ref_stddev_f32(x.ctypes.data, c["w"], c["h"], c["stride"], m.ctypes.data)
        out["stddev_f32"].append(dict(case=c, mean=cases.bits(m)[0], std=cases.bits([s])[0]))
        x = cases.stat_input_f16(c)
        s = R.ref_stddev_f16(x.ctypes.data, c["w"], c["h"], c["stride"], m.ctypes.data)
        out["stddev_f16"].append(dict(case=c, mean=cases.bits(m)[0], std=cases.bits([s])[0]))

    for c in cases.MEDIAN_CASES:
        x = cases.median_input(c)
        o = np.zeros_like(x)
        mn = R.ref_median_filter(x.ctypes.data, o.ctypes.data, c["size"], c["window"])
        out["median"].append(dict(case=c, out_sha=cases.sha(o), mean=cases.bits([mn])[0]))

    for c in cases.SMOOTH_CASES:
        dd = cases.smooth_input(c)
        ndms, ntd = dd.shape
        nbox, sm = 0, c["wmin"]
        while sm < c["wmax"]:
            nbox, sm = nbox + 1, sm * 2
        boxes = np.zeros((nbox, ndms - 2, c["ntime_out"]), np.float32)
        taps = np.zeros(100000, np.float32)
        R.ref_smooth(dd.ctypes.data, ndms, ntd, c["ntime_out"], c["wmin"], c["wmax"], boxes.ctypes.data,
                     taps.ctypes.data, taps.size)
        ntaps = sum(3 * (2 * (c["wmin"] << b) + 1) for b in range(nbox))
        cap = 10000
        snr, wd, dm, sp = (np.zeros(cap, np.float32), np.zeros(cap, np.int32), np.zeros(cap, np.int32),
                           np.zeros(cap, np.int32))
        n = R.ref_find_peaks(boxes.ctypes.data, nbox, ndms, c["ntime_out"], c["snr"], 0, snr.ctypes.data,
                             wd.ctypes.data, dm.ctypes.data, sp.ctypes.data)
        out["smooth"].append(dict(case=c, boxes_sha=cases.sha(boxes), taps=cases.bits(taps[:ntaps]), npeaks=int(n),
                                  peaks_sha=cases.sha(np.stack([snr[:n].view(np.int32), wd[:n], dm[:n], sp[:n]])),
                                  peaks_head=[[int(a), int(b), int(d), cases.bits([v])[0]]
                                              for v, a, b, d in zip(snr[:8], wd[:8], dm[:8], sp[:8])]))
    (HERE / "reference_fixtures.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "reference_fixtures.json")


if __name__ == "__main__":
    main()
