"""ctypes binding of the CPU oracle (oracle/build/libhella_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
benchmark's CPU-baseline leg, to compare the GPU path against.  Never used by the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "libhella_oracle.so"

_lib = None


class Scrunch(C.Structure):
    _fields_ = [("tscrunch", C.c_int), ("fscrunch", C.c_int), ("nits", C.c_int), ("thresh", C.c_float)]


class FlagParams(C.Structure):
    _fields_ = [("spec_min", C.c_float), ("spec_max", C.c_float), ("flag1", C.c_int), ("flag2", C.c_int),
                ("nscrunch", C.c_int), ("scrunches", C.POINTER(Scrunch)), ("bp_median", C.c_int)]


class FlagTrace(C.Structure):
    _fields_ = [("bp1", C.c_float * 8192), ("mean1", C.c_float), ("std1", C.c_float),
                ("bp2", C.c_float * 8192), ("bp3", C.c_float * 8192), ("mean2", C.c_float),
                ("std2", C.c_float)]


class Params(C.Structure):
    _fields_ = [("nchan", C.c_int), ("nbeam", C.c_int), ("gulp", C.c_int), ("tsamp_s", C.c_double),
                ("plan_dt", C.c_double), ("f0_mhz", C.c_double), ("df_mhz", C.c_double),
                ("dm_min", C.c_float), ("dm_max", C.c_float), ("dm_tol", C.c_float), ("ti_us", C.c_float),
                ("wmin", C.c_int), ("wmax", C.c_int), ("snr", C.c_float), ("max_giants", C.c_int),
                ("smooth_anchor", C.c_int), ("flag", FlagParams), ("always_find_peaks", C.c_int)]


class Cand(C.Structure):
    _fields_ = [("beam", C.c_int32), ("dm_idx", C.c_int32), ("width", C.c_int32), ("samp", C.c_int32),
                ("snr", C.c_float)]


CAND_DTYPE = np.dtype([("beam", "<i4"), ("dm_idx", "<i4"), ("width", "<i4"), ("samp", "<i4"),
                       ("snr", "<f4")])
_VP = C.c_void_p


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.ho_f2h.restype = C.c_uint16
        L.ho_f2h.argtypes = [C.c_float]
        L.ho_h2f.restype = C.c_float
        L.ho_h2f.argtypes = [C.c_uint16]
        for n in ("ho_hadd", "ho_hmul", "ho_hdiv"):
            getattr(L, n).restype = C.c_uint16
            getattr(L, n).argtypes = [C.c_uint16, C.c_uint16]
        L.ho_generate_dm_list.argtypes = [_VP, C.c_int] + [C.c_double] * 4 + [C.c_int] + [C.c_double] * 3
        L.ho_delay_table.argtypes = [_VP, C.c_int, C.c_double, C.c_double, C.c_double]
        L.ho_dm_delays.argtypes = [_VP, _VP, C.c_int, _VP, C.c_int]
        L.ho_dedisperse.argtypes = [_VP, C.c_int, C.c_size_t, C.c_int, _VP, C.c_int, _VP, _VP, C.c_size_t,
                                    C.c_int]
        L.ho_stddev_f32.restype = C.c_float
        L.ho_stddev_f32.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, _VP]
        L.ho_stddev_f16.restype = C.c_float
        L.ho_stddev_f16.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, _VP]
        L.ho_flag_beam.argtypes = [_VP, C.c_int, C.c_int, C.POINTER(FlagParams), _VP, _VP, _VP, _VP]
        L.ho_smooth_taps.restype = C.c_int
        L.ho_smooth_taps.argtypes = [C.c_int, _VP]
        L.ho_smooth_plane.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int, _VP,
                                      C.c_int, C.c_size_t]
        L.ho_smooth_normalise.restype = C.c_int
        L.ho_smooth_normalise.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                          C.c_int, _VP, _VP, _VP]
        L.ho_find_peaks.restype = C.c_int
        L.ho_find_peaks.argtypes = [_VP, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, _VP, _VP]
        L.ho_pipeline_create.restype = _VP
        L.ho_pipeline_create.argtypes = [C.POINTER(Params)]
        L.ho_pipeline_destroy.argtypes = [_VP]
        L.ho_pipeline_info.argtypes = [_VP] + [C.POINTER(C.c_int)] * 6
        L.ho_pipeline_dms.restype = C.POINTER(C.c_float)
        L.ho_pipeline_dms.argtypes = [_VP]
        L.ho_pipeline_delays.restype = C.POINTER(C.c_int32)
        L.ho_pipeline_delays.argtypes = [_VP]
        L.ho_pipeline_gulp.restype = C.c_int
        L.ho_pipeline_gulp.argtypes = [_VP, _VP, _VP, C.c_int, C.POINTER(C.c_int)]
        L.ho_pipeline_gulp_f16.restype = C.c_int
        L.ho_pipeline_gulp_f16.argtypes = [_VP, _VP, _VP, C.c_int, C.POINTER(C.c_int)]
        L.ho_flag_beam_f16.argtypes = [_VP, C.c_int, C.c_int, C.POINTER(FlagParams), _VP, _VP, _VP, _VP]
        L.ho_pipeline_ring.restype = C.POINTER(C.c_uint8)
        L.ho_pipeline_ring.argtypes = [_VP, C.c_int]
        L.ho_pipeline_flagspec.restype = C.POINTER(C.c_float)
        L.ho_pipeline_flagspec.argtypes = [_VP]
        L.ho_pipeline_set_killmask.restype = C.c_int
        L.ho_pipeline_set_killmask.argtypes = [_VP, C.c_int, _VP]
        L.ho_search_window.restype = C.c_int
        L.ho_search_window.argtypes = [_VP, _VP, C.c_int, C.c_int, _VP, _VP, _VP, _VP, _VP, _VP]
        L.ho_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().ho_set_threads(n)


# --------------------------------------------------------------- wrappers

def f16(x: float) -> int:
    return lib().ho_f2h(x)


def dm_list(dm_start, dm_end, ti_us, tol, nchan, dt, f0, df) -> np.ndarray:
    buf = np.zeros(1 << 20, np.float32)
    n = lib().ho_generate_dm_list(buf.ctypes.data, buf.size, dm_start, dm_end, ti_us, tol, nchan, dt, f0, df)
    assert n > 0
    return buf[:n].copy()


def delay_table(nchan, dt, f0, df) -> np.ndarray:
    t = np.zeros(nchan, np.float32)
    lib().ho_delay_table(t.ctypes.data, nchan, dt, f0, df)
    return t


def dm_delays(dms, table) -> np.ndarray:
    dms = np.ascontiguousarray(dms, np.float32)
    table = np.ascontiguousarray(table, np.float32)
    out = np.zeros((dms.size, table.size), np.int32)
    lib().ho_dm_delays(out.ctypes.data, dms.ctypes.data, dms.size, table.ctypes.data, table.size)
    return out


def dedisperse(data: np.ndarray, delays: np.ndarray, killmask=None, nout=None) -> np.ndarray:
    data = np.ascontiguousarray(data, np.uint8)
    delays = np.ascontiguousarray(delays, np.int32)
    nsamps, nchan = data.shape
    ndms = delays.shape[0]
    nout = nsamps - int(delays.max()) if nout is None else nout
    km = None if killmask is None else np.ascontiguousarray(killmask, np.int32)
    out = np.zeros((ndms, nout), np.float32)
    lib().ho_dedisperse(data.ctypes.data, nsamps, nchan, nchan, delays.ctypes.data, ndms,
                        None if km is None else km.ctypes.data, out.ctypes.data, nout, nout)
    return out


def stddev_f32(x: np.ndarray, width=None):
    x = np.ascontiguousarray(x, np.float32)
    m = np.zeros(1, np.float32)
    s = lib().ho_stddev_f32(x.ctypes.data, x.shape[1] if width is None else width, x.shape[0], x.shape[1],
                            m.ctypes.data)
    return float(m[0]), float(s)


def flag_params(spec_min=-0.05, spec_max=0.15, flag1=-1, flag2=-1, scrunches=(), bp_median=1):
    arr = (Scrunch * max(1, len(scrunches)))(*[Scrunch(t, f, n, th) for (t, f, th, n) in scrunches])
    fp = FlagParams(spec_min, spec_max, flag1, flag2, len(scrunches), arr, bp_median)
    fp._keep = arr
    return fp


def flag_beam(gulp: np.ndarray, fp: FlagParams | None = None, flagspec=None):
    """u8 [w][nchan] -> (u8 [w][nchan], ts [w], trace dict)."""
    gulp = np.ascontiguousarray(gulp, np.uint8)
    w, nchan = gulp.shape
    fp = fp or flag_params()
    out = np.zeros_like(gulp)
    ts = np.zeros(w, np.float32)
    tr = FlagTrace()
    lib().ho_flag_beam(gulp.ctypes.data, w, nchan, C.byref(fp), out.ctypes.data, ts.ctypes.data,
                       None if flagspec is None else flagspec.ctypes.data, C.byref(tr))
    trace = dict(bp1=np.array(tr.bp1[:nchan], np.float32), bp2=np.array(tr.bp2[:nchan], np.float32),
                 bp3=np.array(tr.bp3[:nchan], np.float32), mean1=np.float32(tr.mean1),
                 std1=np.float32(tr.std1), mean2=np.float32(tr.mean2), std2=np.float32(tr.std2))
    return out, ts, trace


def flag_beam_f16(ft: np.ndarray, fp: FlagParams | None = None, flagspec=None):
    """fp16 channel-major [nchan][w] (the DADA input) -> (u8 [w][nchan], ts [w], trace dict)."""
    ft = np.ascontiguousarray(ft, np.float16)
    nchan, w = ft.shape
    fp = fp or flag_params()
    out = np.zeros((w, nchan), np.uint8)
    ts = np.zeros(w, np.float32)
    tr = FlagTrace()
    lib().ho_flag_beam_f16(ft.ctypes.data, w, nchan, C.byref(fp), out.ctypes.data, ts.ctypes.data,
                           None if flagspec is None else flagspec.ctypes.data, C.byref(tr))
    trace = dict(bp1=np.array(tr.bp1[:nchan], np.float32), bp2=np.array(tr.bp2[:nchan], np.float32),
                 bp3=np.array(tr.bp3[:nchan], np.float32), mean1=np.float32(tr.mean1),
                 std1=np.float32(tr.std1), mean2=np.float32(tr.mean2), std2=np.float32(tr.std2))
    return out, ts, trace


def box_filter(plane: np.ndarray, xw: int, yw: int, k: float) -> np.ndarray:
    """The SCRUNCH box filter (convolution.cu:20-55) on an fp16 plane given as
    uint16 bit patterns [nchan][w]."""
    plane = np.ascontiguousarray(plane, np.uint16)
    out = np.zeros_like(plane)
    L = lib()
    L.ho_box_filter.argtypes = [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float]
    L.ho_box_filter(plane.ctypes.data, out.ctypes.data, plane.shape[0], plane.shape[1], xw, yw, k)
    return out


def smooth_plane(dd: np.ndarray, sm: int, wmax: int, ntime_out: int, anchor: int = 1,
                 direct: bool = False) -> np.ndarray:
    """One width's pre-normalisation plane [ndms-2][ntime_out]: the factored
    form (ho_smooth_plane), or the kernel tap by tap (ho_smooth_plane_direct)."""
    dd = np.ascontiguousarray(dd, np.float32)
    ndms, ntd = dd.shape
    out = np.zeros((ndms - 2, ntime_out), np.float32)
    L = lib()
    f = L.ho_smooth_plane_direct if direct else L.ho_smooth_plane
    f.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int, _VP, C.c_int, C.c_size_t]
    f(dd.ctypes.data, ndms, ntd, ntd, sm, wmax, 2 * sm if anchor else 0, out.ctypes.data, ntime_out, ntime_out)
    return out


def smooth_taps(sm: int) -> np.ndarray:
    k = np.zeros(3 * (2 * sm + 1), np.float32)
    lib().ho_smooth_taps(sm, k.ctypes.data)
    return k.reshape(3, 2 * sm + 1)


class Pipeline:
    """The oracle gulp loop (casm_hella_refactored.cu:659-835)."""

    def __init__(self, *, nchan, nbeam, gulp, tsamp, plan_dt, f0, df, dm_min, dm_max, dm_tol, ti_us, wmin,
                 wmax, snr, max_giants=10000, anchor=0, spec_min=-0.05, spec_max=0.15, flag1=-1, flag2=-1,
                 scrunches=(), bp_median=1, always_find_peaks=0):
        self.fp = flag_params(spec_min, spec_max, flag1, flag2, scrunches, bp_median)
        self.p = Params(nchan, nbeam, gulp, tsamp, plan_dt, f0, df, dm_min, dm_max, dm_tol, ti_us, wmin, wmax,
                        snr, max_giants, anchor, self.fp, always_find_peaks)
        self.L = lib()
        self.h = self.L.ho_pipeline_create(C.byref(self.p))
        if not self.h:
            raise ValueError("oracle pipeline creation failed")
        v = [C.c_int() for _ in range(6)]
        self.L.ho_pipeline_info(self.h, *[C.byref(x) for x in v])
        self.ntime, self.ndms, self.max_delay, self.ntime_dd, self.nbox, self.min_gulp = [x.value for x in v]
        self.nchan, self.nbeam, self.gulp, self.max_giants = nchan, nbeam, gulp, max_giants

    @classmethod
    def from_params(cls, params: dict, **over) -> "Pipeline":
        """From the product's parameter names (hella_params fields)."""
        p = dict(params)
        p.update(over)
        return cls(nchan=p["nchan"], nbeam=p.get("nbeam", 1), gulp=p["gulp"], tsamp=p["tsamp"],
                   plan_dt=p["plan_dt"], f0=p["f0_mhz"], df=p["df_mhz"], dm_min=p["dm_min"], dm_max=p["dm_max"],
                   dm_tol=p["dm_tol"], ti_us=p["ti_us"], wmin=p["width_min"], wmax=p["width_max"], snr=p["snr"],
                   max_giants=p.get("max_giants", 10000), anchor=p.get("smooth_anchor", 1),
                   spec_min=p.get("spec_min", -0.05), spec_max=p.get("spec_max", 0.15), flag1=p.get("flag1", -1),
                   flag2=p.get("flag2", -1), scrunches=p.get("scrunches", ()), bp_median=p.get("bp_median", 1),
                   always_find_peaks=p.get("always_find_peaks", 0))

    def close(self):
        if getattr(self, "h", None):
            self.L.ho_pipeline_destroy(self.h)
            self.h = None

    __del__ = close

    def dms(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ho_pipeline_dms(self.h), shape=(self.ndms,)).copy()

    def delays(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ho_pipeline_delays(self.h), shape=(self.ndms, self.nchan)).copy()

    def ring(self, beam: int) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ho_pipeline_ring(self.h, beam), shape=(self.ntime, self.nchan)).copy()

    def flagspec(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ho_pipeline_flagspec(self.h), shape=(self.nchan,)).copy()

    def set_killmask(self, beam: int, killmask):
        """Beam `beam`'s dedispersion killmask (0 drops a channel; None: all kept)."""
        km = None if killmask is None else np.ascontiguousarray(killmask, np.int32)
        if km is not None and km.shape != (self.nchan,):
            raise ValueError("killmask needs one entry per channel")
        if self.L.ho_pipeline_set_killmask(self.h, beam, None if km is None else km.ctypes.data) != 0:
            raise ValueError("beam outside the pipeline")

    def gulp_step(self, gulp: np.ndarray):
        gulp = np.ascontiguousarray(gulp, np.uint8)
        out = np.zeros(self.max_giants, CAND_DTYPE)
        s = C.c_int()
        n = self.L.ho_pipeline_gulp(self.h, gulp.ctypes.data, out.ctypes.data, self.max_giants, C.byref(s))
        return out[:n], bool(s.value)

    def gulp_step_f16(self, gulp: np.ndarray):
        """One gulp of fp16 FT data [nbeam][nchan][gulp] (DADA input)."""
        gulp = np.ascontiguousarray(gulp, np.float16)
        out = np.zeros(self.max_giants, CAND_DTYPE)
        s = C.c_int()
        n = self.L.ho_pipeline_gulp_f16(self.h, gulp.ctypes.data, out.ctypes.data, self.max_giants, C.byref(s))
        return out[:n], bool(s.value)

    def search_window(self, window: np.ndarray, beam=0, cap=None, want_planes=True):
        window = np.ascontiguousarray(window, np.uint8)
        cap = self.max_giants if cap is None else cap
        out = np.zeros(cap, CAND_DTYPE)
        dd = np.zeros((self.ndms, self.ntime_dd), np.float32) if want_planes else None
        bx = np.zeros((self.nbox, self.ndms - 2, self.gulp), np.float32) if want_planes else None
        mean, std, s0 = np.zeros(self.nbox, np.float32), np.zeros(self.nbox, np.float32), np.zeros(1, np.float32)
        n = self.L.ho_search_window(self.h, window.ctypes.data, beam, cap, out.ctypes.data,
                                    None if dd is None else dd.ctypes.data, None if bx is None else bx.ctypes.data,
                                    mean.ctypes.data, std.ctypes.data, s0.ctypes.data)
        return dict(cands=out[:n], dd=dd, boxes=bx, mean=mean, std=std, sigma0=float(s0[0]))


def stddev_f16(x: np.ndarray, width=None):
    """calculate_stddev<half> of an fp16 plane given as uint16 bit patterns."""
    x = np.ascontiguousarray(x, np.uint16)
    m = np.zeros(1, np.float32)
    s = lib().ho_stddev_f16(x.ctypes.data, x.shape[1] if width is None else width, x.shape[0], x.shape[1],
                            m.ctypes.data)
    return float(m[0]), float(s)


def median_filter(x: np.ndarray, window: int):
    L = lib()
    L.ho_median_filter.restype = C.c_float
    L.ho_median_filter.argtypes = [_VP, _VP, C.c_int, C.c_int]
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    mn = L.ho_median_filter(x.ctypes.data, out.ctypes.data, x.size, window)
    return out, float(mn)


def smooth_normalise(dd: np.ndarray, wmin: int, wmax: int, ntime_out: int, anchor: int = 1, direct: bool = False):
    """smooth(p, 1): (standardised planes, means, stds).  direct: the kernel
    applied tap by tap (the emulator's NPP stand-in) instead of the factored
    form the GPU computes."""
    dd = np.ascontiguousarray(dd, np.float32)
    ndms, ntd = dd.shape
    nbox, sm = 0, wmin
    while sm < wmax:
        nbox, sm = nbox + 1, sm * 2
    boxes = np.zeros((nbox, ndms - 2, ntime_out), np.float32)
    mean, std = np.zeros(nbox, np.float32), np.zeros(nbox, np.float32)
    L = lib()
    L.ho_smooth_normalise_arith.argtypes = [_VP, C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int,
                                            _VP, _VP, _VP, C.c_int]
    L.ho_smooth_normalise_arith(dd.ctypes.data, ndms, ntd, ntd, wmin, wmax, anchor, ntime_out, boxes.ctypes.data,
                                mean.ctypes.data, std.ctypes.data, int(direct))
    return boxes, mean, std


def find_peaks(boxes: np.ndarray, snr: float, beam: int = 0, cap: int = 10000, gate: bool = True):
    boxes = np.ascontiguousarray(boxes, np.float32)
    nbox, h, nt = boxes.shape
    out = np.zeros(cap, CAND_DTYPE)
    s0 = np.zeros(1, np.float32)
    L = lib()
    L.ho_find_peaks_gate.restype = C.c_int
    L.ho_find_peaks_gate.argtypes = [_VP, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, _VP, _VP, C.c_int]
    n = L.ho_find_peaks_gate(boxes.ctypes.data, nbox, h + 2, nt, snr, beam, cap, out.ctypes.data, s0.ctypes.data,
                             int(gate))
    return out[:n], float(s0[0])
