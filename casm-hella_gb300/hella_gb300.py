"""ctypes binding of libhella_gb300.so (include/hella_dedisp.h, hella_search.h).

A thin mirror of the C ABI for the Python test harness and the benchmark.
Loading fails loudly when the library has not been built: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libhella_gb300.so"

_lib = None

# --------------------------------------------------------------- structures

HELLA_MAX_SCRUNCH = 16
HELLA_MAX_GIANTS = 10000

HDD_HOST_POINTERS = 1 << 1
HDD_DEVICE_POINTERS = 1 << 2
HDD_WAIT = 1 << 3
HDD_ASYNC = 1 << 4

HDD_ERRORS = [
    "HDD_NO_ERROR", "HDD_MEM_ALLOC_FAILED", "HDD_MEM_COPY_FAILED", "HDD_NCHANS_EXCEEDS_LIMIT",
    "HDD_INVALID_PLAN", "HDD_INVALID_POINTER", "HDD_INVALID_STRIDE", "HDD_NO_DM_LIST_SET",
    "HDD_TOO_FEW_NSAMPS", "HDD_INVALID_FLAG_COMBINATION", "HDD_UNSUPPORTED_IN_NBITS",
    "HDD_UNSUPPORTED_OUT_NBITS", "HDD_INVALID_DEVICE_INDEX", "HDD_DEVICE_ALREADY_SET",
    "HDD_PRIOR_GPU_ERROR", "HDD_INTERNAL_GPU_ERROR", "HDD_UNKNOWN_ERROR", "HDD_STATIC_SCRATCH_EXCEEDED",
]


class HellaScrunch(C.Structure):
    _fields_ = [("tscrunch", C.c_int), ("fscrunch", C.c_int), ("nits", C.c_int), ("thresh", C.c_float)]


class HellaParams(C.Structure):
    _fields_ = [
        ("nchan", C.c_int), ("nbeam", C.c_int), ("gulp", C.c_int),
        ("tsamp", C.c_double), ("plan_dt", C.c_double), ("f0_mhz", C.c_double), ("df_mhz", C.c_double),
        ("dm_min", C.c_float), ("dm_max", C.c_float), ("dm_tol", C.c_float), ("ti_us", C.c_float),
        ("width_min", C.c_int), ("width_max", C.c_int), ("snr", C.c_float),
        ("spec_min", C.c_float), ("spec_max", C.c_float), ("flag1", C.c_int), ("flag2", C.c_int),
        ("nscrunch", C.c_int), ("scrunch", HellaScrunch * HELLA_MAX_SCRUNCH),
        ("max_giants", C.c_int), ("beam0", C.c_int), ("smooth_anchor", C.c_int), ("device", C.c_int),
        ("hbm_budget", C.c_size_t), ("autotune", C.c_int), ("input_format", C.c_int), ("bp_median", C.c_int),
        ("always_find_peaks", C.c_int),
    ]


class BatchParams(C.Structure):
    _fields_ = [("base", HellaParams), ("dm_max", C.c_void_p), ("killmask", C.c_void_p),
                ("widths_per_pass", C.c_int), ("use_graph", C.c_int), ("dynamic", C.c_int),
                ("member", C.c_void_p), ("inflight", C.c_int), ("bp_alpha", C.c_float)]


class FilHeader(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("machine_id", "telescope_id", "data_type", "nchans", "nbits", "nifs",
                                        "barycentric", "pulsarcentric", "ibeam", "nbeams")] + \
               [(k, C.c_double) for k in ("tstart", "tsamp", "fch1", "foff", "refdm", "az_start", "za_start",
                                          "src_raj", "src_dej", "period")] + \
               [("isign", C.c_char), ("npuls", C.c_long), ("source_name", C.c_char * 81),
                ("rawdatafile", C.c_char * 81), ("nfreq", C.c_int), ("header_bytes", C.c_long),
                ("frequency_table", C.c_double * 4096)]


class RefineParams(C.Structure):
    _fields_ = [("ncut", C.c_int), ("nchan", C.c_int), ("nsamp", C.c_int), ("tsamp", C.c_double),
                ("f0_mhz", C.c_double), ("df_mhz", C.c_double), ("device", C.c_int)]


class PairTablesView(C.Structure):
    """hdd_pair_tables_view: host group-row tables of a plan (tests)."""
    _fields_ = [("channels", C.c_int), ("stage_groups", C.c_int), ("time_tiles", C.c_int), ("ntiles", C.c_int),
                ("ngroups", C.c_int), ("nrows", C.c_int), ("nrec", C.c_int), ("rec_ints", C.c_int),
                ("max_stage_bytes", C.c_int), ("max_span", C.c_int), ("npos", C.c_long), ("words", C.c_long),
                ("rinfo", C.POINTER(C.c_int)), ("rinfo2", C.POINTER(C.c_int)), ("roff", C.POINTER(C.c_longlong)),
                ("rwords", C.POINTER(C.c_int)), ("rtile", C.POINTER(C.c_int)), ("prow", C.POINTER(C.c_int)),
                ("prange", C.POINTER(C.c_int)),
                ("rec", C.POINTER(C.c_int)), ("tile_st", C.POINTER(C.c_int))]


class HellaTuning(C.Structure):
    _fields_ = [("dm_per_block", C.c_int), ("samples_per_thread", C.c_int), ("chan_chunk", C.c_int),
                ("stages", C.c_int), ("group", C.c_int), ("add_mode", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class HellaInfo(C.Structure):
    _fields_ = [
        ("ntime", C.c_int), ("ndms", C.c_int), ("max_delay", C.c_int), ("ntime_dd", C.c_int),
        ("ntime_out", C.c_int), ("nboxcar", C.c_int), ("min_gulp", C.c_int), ("gulp_index", C.c_int),
        ("device_bytes", C.c_size_t),
    ]


class HellaCand(C.Structure):
    _fields_ = [("beam", C.c_int32), ("dm_idx", C.c_int32), ("width", C.c_int32),
                ("samp", C.c_int32), ("snr", C.c_float)]


CAND_DTYPE = np.dtype([("beam", "<i4"), ("dm_idx", "<i4"), ("width", "<i4"), ("samp", "<i4"),
                       ("snr", "<f4")])

# ------------------------------------------------------------------ loading

_VP = C.c_void_p
_SZ = C.c_ulong


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with casm-hella_gb300/build.py")
    L = C.CDLL(str(LIB_PATH))
    # hdd_ plan API
    _sig(L, "hdd_create_plan", C.c_int, [C.POINTER(_VP), _SZ, C.c_float, C.c_float, C.c_float])
    _sig(L, "hdd_destroy_plan", None, [_VP])
    _sig(L, "hdd_set_device", C.c_int, [C.c_int])
    _sig(L, "hdd_set_stream", C.c_int, [_VP, _VP])
    _sig(L, "hdd_set_pair_rows", C.c_int, [_VP, C.c_int])
    _sig(L, "hdd_set_dm_list", C.c_int, [_VP, _VP, _SZ])
    _sig(L, "hdd_generate_dm_list", C.c_int, [_VP, C.c_float, C.c_float, C.c_float, C.c_float])
    _sig(L, "hdd_set_killmask", C.c_int, [_VP, _VP])
    for n in ("hdd_get_max_delay", "hdd_get_channel_count", "hdd_get_dm_count"):
        _sig(L, n, _SZ, [_VP])
    _sig(L, "hdd_get_dm_delay", _SZ, [_VP, C.c_int])
    _sig(L, "hdd_get_dm_list", C.POINTER(C.c_float), [_VP])
    _sig(L, "hdd_get_killmask", C.POINTER(C.c_int), [_VP])
    _sig(L, "hdd_get_delay_table", C.POINTER(C.c_int), [_VP])
    _sig(L, "hdd_get_pair_tables", C.c_int, [_VP, C.c_size_t, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                             C.POINTER(PairTablesView)])
    for n in ("hdd_get_dt", "hdd_get_df", "hdd_get_f0"):
        _sig(L, n, C.c_float, [_VP])
    _sig(L, "hdd_execute", C.c_int, [_VP, _SZ, _VP, _SZ, _VP, _SZ, C.c_uint])
    _sig(L, "hdd_execute_adv", C.c_int, [_VP, _SZ, _VP, _SZ, _SZ, _VP, _SZ, _SZ, C.c_uint])
    _sig(L, "hdd_execute_guru", C.c_int, [_VP, _SZ, _VP, _SZ, _SZ, _VP, _SZ, _SZ, _SZ, _SZ, C.c_uint])
    _sig(L, "hdd_get_error_string", C.c_char_p, [C.c_int])
    _sig(L, "hdd_execute_noalloc", C.c_int, [_VP, _SZ, _VP, _SZ, _SZ, _VP, _SZ, _SZ, C.c_uint])
    # hella_ stage API
    _sig(L, "hella_params_default", None, [C.POINTER(HellaParams)])
    _sig(L, "hella_create", C.c_int, [C.POINTER(_VP), C.POINTER(HellaParams)])
    _sig(L, "hella_destroy", None, [_VP])
    _sig(L, "hella_set_stream", C.c_int, [_VP, _VP])
    _sig(L, "hella_get_info", C.c_int, [_VP, C.POINTER(HellaInfo)])
    _sig(L, "hella_get_dm_list", C.POINTER(C.c_float), [_VP])
    _sig(L, "hella_set_killmask", C.c_int, [_VP, _VP])
    _sig(L, "hella_load_gulp", C.c_int, [_VP, _VP, C.c_int])
    for n in ("hella_fast_flagger", "hella_clear_peaks", "hella_rewind"):
        _sig(L, n, C.c_int, [_VP])
    for n in ("hella_dedisperse", "hella_smooth", "hella_find_peaks"):
        _sig(L, n, C.c_int, [_VP, C.c_int])
    _sig(L, "hella_get_peaks", C.c_int, [_VP, _VP, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "hella_process_gulp", C.c_int,
         [_VP, _VP, C.c_int, _VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)])
    _sig(L, "hella_copy_window", C.c_int, [_VP, C.c_int, _VP])
    _sig(L, "hella_copy_dedisp", C.c_int, [_VP, _VP])
    _sig(L, "hella_copy_boxes", C.c_int, [_VP, _VP])
    _sig(L, "hella_get_smooth_stats", C.c_int, [_VP, _VP, _VP, _VP])
    _sig(L, "hella_get_flag_stats", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, _VP])
    _sig(L, "hella_get_flag_spec", C.c_int, [_VP, _VP])
    _sig(L, "hella_status_string", C.c_char_p, [C.c_int])
    _sig(L, "hella_batch_params_default", None, [C.POINTER(BatchParams)])
    _sig(L, "hella_batch_create", C.c_int, [C.POINTER(_VP), C.POINTER(BatchParams)])
    _sig(L, "hella_batch_destroy", None, [_VP])
    _sig(L, "hella_batch_set_stream", C.c_int, [_VP, _VP])
    _sig(L, "hella_batch_get_info", C.c_int, [_VP, C.c_int, C.POINTER(HellaInfo)])
    _sig(L, "hella_batch_process_gulp", C.c_int, [_VP, _VP, C.c_int, _VP, C.c_int, C.POINTER(C.c_int), _VP, _VP])
    _sig(L, "hella_batch_copy_dedisp", C.c_int, [_VP, C.c_int, _VP])
    _sig(L, "hella_batch_get_tuning", C.c_int, [_VP, C.POINTER(HellaTuning)])
    _sig(L, "hella_batch_set_tuning", C.c_int, [_VP, C.POINTER(HellaTuning)])
    _sig(L, "hella_batch_time_dedisp", C.c_int, [_VP, C.POINTER(HellaTuning), C.c_int, C.POINTER(C.c_float)])
    _sig(L, "hella_batch_autotune", C.c_int, [_VP, C.c_int, C.POINTER(HellaTuning), C.POINTER(C.c_float)])
    _sig(L, "hella_batch_last_gulp_ms", C.c_int, [_VP, C.POINTER(C.c_float)])
    _sig(L, "hella_batch_graph_kernels", C.c_int, [_VP, C.POINTER(C.c_int)])
    _sig(L, "hella_batch_submit", C.c_int, [_VP, _VP, C.c_int])
    _sig(L, "hella_batch_poll", C.c_int, [_VP, _VP, C.c_int, C.POINTER(C.c_int), _VP, _VP,
                                           C.POINTER(C.c_float), C.POINTER(C.c_float)])
    _sig(L, "hella_batch_set_beam", C.c_int, [_VP, C.c_int, C.c_int, C.c_float, _VP])
    _sig(L, "hella_batch_get_bandpass", C.c_int, [_VP, C.c_int, _VP])
    _sig(L, "hella_batch_get_flag_spec", C.c_int, [_VP, _VP])
    _sig(L, "hella_batch_bytes", C.c_int, [C.POINTER(BatchParams), C.POINTER(C.c_size_t)])
    _sig(L, "hella_refine_create", C.c_int, [C.POINTER(_VP), C.POINTER(RefineParams)])
    _sig(L, "hella_refine_destroy", None, [_VP])
    _sig(L, "hella_refine_set_stream", C.c_int, [_VP, _VP])
    _sig(L, "hella_refine_delay_table", C.c_int, [_VP, _VP])
    _sig(L, "hella_refine_forward", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP])
    _sig(L, "hella_refine_adjoint", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, _VP])
    _sig(L, "hella_refine_fit", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, C.c_int, _VP, _VP])
    # I/O around the search
    _sig(L, "hella_fil_open", C.c_int, [C.POINTER(_VP), C.c_char_p, C.c_int, C.POINTER(FilHeader)])
    _sig(L, "hella_fil_read", C.c_int, [_VP, _VP, C.c_int, C.POINTER(C.c_int)])
    _sig(L, "hella_fil_close", None, [_VP])
    _sig(L, "hella_cands_format", C.c_int, [_VP, C.c_int, C.c_long, _VP, C.c_int, C.c_double, _VP, C.c_size_t,
                                            C.POINTER(C.c_size_t)])
    _sig(L, "hella_cands_append", C.c_int, [C.c_char_p, _VP, C.c_int, C.c_long, _VP, C.c_int, C.c_double])
    _sig(L, "hella_cands_coincidencer", C.c_int, [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, _VP, C.c_int,
                                                  C.c_long, _VP, C.c_int, C.c_double, _VP, C.c_size_t,
                                                  C.POINTER(C.c_size_t)])
    _sig(L, "hella_cands_send", C.c_int, [C.c_char_p, C.c_int, C.c_char_p, C.c_size_t, C.c_int])
    _sig(L, "hella_cluster", C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, _VP, C.POINTER(C.c_int), _VP])
    _sig(L, "hella_flagstats_create", C.c_int, [C.POINTER(_VP), C.c_int, C.c_int])
    _sig(L, "hella_flagstats_destroy", None, [_VP])
    _sig(L, "hella_flagstats_update", C.c_int, [_VP, _VP])
    _sig(L, "hella_flagstats_counts", C.c_int, [_VP, _VP])
    _sig(L, "hella_flagstats_append", C.c_int, [_VP, C.c_char_p])
    _sig(L, "hella_ring_create", C.c_int, [C.POINTER(_VP), C.c_size_t, C.c_int, C.c_int])
    _sig(L, "hella_ring_destroy", None, [_VP])
    _sig(L, "hella_ring_block_bytes", C.c_size_t, [_VP])
    _sig(L, "hella_ring_write_header", C.c_int, [_VP, C.c_char_p, C.c_size_t])
    _sig(L, "hella_ring_read_header", C.c_int, [_VP, _VP, C.c_size_t, C.POINTER(C.c_size_t), C.c_int])
    _sig(L, "hella_ring_open_write", C.c_int, [_VP, C.POINTER(_VP), C.c_int])
    _sig(L, "hella_ring_mark_filled", C.c_int, [_VP, C.c_size_t])
    _sig(L, "hella_ring_end", C.c_int, [_VP])
    _sig(L, "hella_ring_open_read", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(C.c_size_t), C.c_int])
    _sig(L, "hella_ring_mark_cleared", C.c_int, [_VP])
    _sig(L, "hella_header_get", C.c_int, [C.c_char_p, C.c_size_t, C.c_char_p, _VP, C.c_size_t])
    _sig(L, "hella_get_tuning", C.c_int, [_VP, C.POINTER(HellaTuning)])
    _sig(L, "hella_set_tuning", C.c_int, [_VP, C.POINTER(HellaTuning)])
    _sig(L, "hella_time_dedisp", C.c_int, [_VP, C.POINTER(HellaTuning), C.c_int, C.POINTER(C.c_float)])
    _sig(L, "hella_autotune", C.c_int, [_VP, C.c_int, C.POINTER(HellaTuning), C.POINTER(C.c_float)])
    _sig(L, "hella_fp16_selftest", C.c_int, [C.c_int, C.POINTER(C.c_ulonglong), C.POINTER(C.c_uint32)])
    _sig(L, "hella_int_add_peak", C.c_int, [C.c_int, C.POINTER(C.c_double)])
    _sig(L, "hella_smem_read_peak", C.c_int, [C.c_int, C.POINTER(C.c_double)])
    _sig(L, "hella_kernel_launches", C.c_ulonglong, [])
    _lib = L
    return L


class HellaError(RuntimeError):
    pass


def _ptr(a) -> int:
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _chk_hdd(rc: int) -> None:
    if rc != 0:
        raise HellaError(f"{HDD_ERRORS[rc] if rc < len(HDD_ERRORS) else rc}: "
                         f"{lib().hdd_get_error_string(rc).decode()}")


def _chk(rc: int) -> None:
    if rc != 0:
        raise HellaError(f"hella status {rc}: {lib().hella_status_string(rc).decode()}")


def fp16_selftest(device: int = 0):
    """(mismatches, first bad pair) of the device fp16 self-check."""
    n, first = C.c_ulonglong(), C.c_uint32()
    _chk(lib().hella_fp16_selftest(device, C.byref(n), C.byref(first)))
    return n.value, first.value


def int_add_peak(device: int = 0) -> float:
    """Measured 32-bit integer adds per second (register-only chains)."""
    v = C.c_double()
    _chk(lib().hella_int_add_peak(device, C.byref(v)))
    return v.value


def smem_read_peak(device: int = 0) -> float:
    """Measured shared-memory bytes per second read by all SMs (16-byte loads)."""
    v = C.c_double()
    _chk(lib().hella_smem_read_peak(device, C.byref(v)))
    return v.value


def kernel_launches() -> int:
    return int(lib().hella_kernel_launches())


# --------------------------------------------------------------- hdd plan

class Plan:
    """The dedisp-shaped plan (hdd_create_plan ... hdd_destroy_plan)."""

    def __init__(self, nchans: int, dt: float, f0: float, df: float):
        self.L = lib()
        h = _VP()
        _chk_hdd(self.L.hdd_create_plan(C.byref(h), nchans, dt, f0, df))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.hdd_destroy_plan(self.h)
            self.h = None

    __del__ = close

    def generate_dm_list(self, dm_start, dm_end, ti_us, tol):
        _chk_hdd(self.L.hdd_generate_dm_list(self.h, dm_start, dm_end, ti_us, tol))

    def set_dm_list(self, dms):
        a = np.ascontiguousarray(dms, dtype=np.float32)
        _chk_hdd(self.L.hdd_set_dm_list(self.h, a.ctypes.data, a.size))

    def set_killmask(self, mask):
        a = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        _chk_hdd(self.L.hdd_set_killmask(self.h, None if a is None else a.ctypes.data))

    def set_stream(self, stream: int):
        _chk_hdd(self.L.hdd_set_stream(self.h, stream))

    def set_pair_rows(self, channels):
        """0 / False: channel by channel; 2 / True: pair rows; 4: rows of four channels."""
        _chk_hdd(self.L.hdd_set_pair_rows(self.h, int(channels)))

    @property
    def dm_count(self) -> int:
        return int(self.L.hdd_get_dm_count(self.h))

    @property
    def max_delay(self) -> int:
        return int(self.L.hdd_get_max_delay(self.h))

    @property
    def nchans(self) -> int:
        return int(self.L.hdd_get_channel_count(self.h))

    def dm_list(self) -> np.ndarray:
        n = self.dm_count
        p = self.L.hdd_get_dm_list(self.h)
        return np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.float32)

    def delay_table(self) -> np.ndarray:
        p = self.L.hdd_get_delay_table(self.h)
        return np.ctypeslib.as_array(p, shape=(self.dm_count, self.nchans)).copy()

    def pair_tables(self, first: int, count: int, channels: int, stage_groups: int, time_tiles: int) -> dict:
        """Copies of the group-row host tables (hdd_get_pair_tables)."""
        v = PairTablesView()
        _chk_hdd(self.L.hdd_get_pair_tables(self.h, first, count, channels, stage_groups, time_tiles, C.byref(v)))
        a = lambda ptr, n: np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        return dict(channels=v.channels, stage_groups=v.stage_groups, time_tiles=v.time_tiles, ntiles=v.ntiles,
                    ngroups=v.ngroups, nrows=v.nrows, max_stage_bytes=v.max_stage_bytes, max_span=v.max_span,
                    npos=v.npos, words=v.words, rinfo=a(v.rinfo, 4 * v.nrows).reshape(-1, 4),
                    rinfo2=a(v.rinfo2, 4 * v.nrows).reshape(-1, 4), roff=a(v.roff, v.nrows),
                    rwords=a(v.rwords, v.nrows), rtile=a(v.rtile, v.nrows), prow=a(v.prow, v.ngroups + 1),
                    prange=a(v.prange, 6 * v.ngroups).reshape(-1, 3, 2),
                    rec=a(v.rec, v.nrec * v.rec_ints).reshape(v.nrec, v.rec_ints), tile_st=a(v.tile_st, v.ntiles + 1))

    def execute_adv(self, nsamps, inp, in_stride, out, out_stride, flags=HDD_HOST_POINTERS, in_nbits=8,
                    out_nbits=32):
        _chk_hdd(self.L.hdd_execute_adv(self.h, nsamps, _ptr(inp), in_nbits, in_stride, _ptr(out), out_nbits,
                                        out_stride, flags))

    def execute_guru(self, nsamps, inp, in_stride, out, out_stride, first, count, flags=HDD_HOST_POINTERS):
        _chk_hdd(self.L.hdd_execute_guru(self.h, nsamps, _ptr(inp), 8, in_stride, _ptr(out), 32, out_stride,
                                         first, count, flags))

    def dedisperse(self, data: np.ndarray) -> np.ndarray:
        """Host convenience: u8 [nsamps][nchans] -> f32 [ndms][nsamps - max_delay]."""
        data = np.ascontiguousarray(data, dtype=np.uint8)
        nout = data.shape[0] - self.max_delay
        out = np.empty((self.dm_count, nout), np.float32)
        self.execute_adv(data.shape[0], data, data.shape[1], out, nout * 4)
        return out


# ------------------------------------------------------------ hella search

def default_params(**kw) -> HellaParams:
    p = HellaParams()
    lib().hella_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "scrunches":
            p.nscrunch = len(v)
            for i, (t, f, th, n) in enumerate(v):
                p.scrunch[i] = HellaScrunch(t, f, n, th)
            continue
        setattr(p, k, v)
    return p


class Search:
    """One search pipeline (hella_create ... hella_destroy)."""

    def __init__(self, params: HellaParams):
        self.L = lib()
        h = _VP()
        _chk(self.L.hella_create(C.byref(h), C.byref(params)))
        self.h = h
        self.params = params
        self.info = self.get_info()

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_destroy(self.h)
            self.h = None

    __del__ = close

    def get_info(self) -> HellaInfo:
        i = HellaInfo()
        _chk(self.L.hella_get_info(self.h, C.byref(i)))
        return i

    def dm_list(self) -> np.ndarray:
        p = self.L.hella_get_dm_list(self.h)
        return np.ctypeslib.as_array(p, shape=(self.info.ndms,)).copy()

    def set_stream(self, stream: int):
        _chk(self.L.hella_set_stream(self.h, stream))

    def set_killmask(self, mask):
        a = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        _chk(self.L.hella_set_killmask(self.h, None if a is None else a.ctypes.data))

    def load_gulp(self, gulp, on_device=False):
        _chk(self.L.hella_load_gulp(self.h, _ptr(gulp), int(on_device)))

    def fast_flagger(self):
        _chk(self.L.hella_fast_flagger(self.h))

    def dedisperse(self, beam: int):
        _chk(self.L.hella_dedisperse(self.h, beam))

    def smooth(self, scale: int = 1):
        _chk(self.L.hella_smooth(self.h, scale))

    def find_peaks(self, beam: int):
        _chk(self.L.hella_find_peaks(self.h, beam))

    def clear_peaks(self):
        _chk(self.L.hella_clear_peaks(self.h))

    def rewind(self):
        _chk(self.L.hella_rewind(self.h))

    def get_peaks(self, max_n: int | None = None) -> np.ndarray:
        max_n = self.params.max_giants if max_n is None else max_n
        out = np.zeros(max_n, CAND_DTYPE)
        n = C.c_int()
        _chk(self.L.hella_get_peaks(self.h, out.ctypes.data, max_n, C.byref(n)))
        return out[: n.value]

    def process_gulp(self, gulp, on_device=False):
        """Returns (candidates, searched)."""
        out = np.zeros(self.params.max_giants, CAND_DTYPE)
        n, s = C.c_int(), C.c_int()
        _chk(self.L.hella_process_gulp(self.h, _ptr(gulp), int(on_device), out.ctypes.data,
                                       self.params.max_giants, C.byref(n), C.byref(s)))
        self.info = self.get_info()
        return out[: n.value], bool(s.value)

    def copy_window(self, beam: int) -> np.ndarray:
        out = np.empty((self.info.ntime, self.params.nchan), np.uint8)
        _chk(self.L.hella_copy_window(self.h, beam, out.ctypes.data))
        return out

    def copy_dedisp(self) -> np.ndarray:
        out = np.empty((self.info.ndms, self.info.ntime_dd), np.float32)
        _chk(self.L.hella_copy_dedisp(self.h, out.ctypes.data))
        return out

    def copy_boxes(self) -> np.ndarray:
        i = self.info
        out = np.empty((i.nboxcar, i.ndms - 2, i.ntime_out), np.float32)
        _chk(self.L.hella_copy_boxes(self.h, out.ctypes.data))
        return out

    def smooth_stats(self):
        n = self.info.nboxcar
        mean, std, s0 = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(1, np.float32)
        _chk(self.L.hella_get_smooth_stats(self.h, mean.ctypes.data, std.ctypes.data, s0.ctypes.data))
        return mean, std, float(s0[0])

    def flag_stats(self, beam: int):
        nch = self.params.nchan
        bp1, bp2, bp3 = (np.zeros(nch, np.float32) for _ in range(3))
        sc = np.zeros(4, np.float32)
        ts = np.zeros(self.params.gulp, np.float32)
        _chk(self.L.hella_get_flag_stats(self.h, beam, bp1.ctypes.data, bp2.ctypes.data, bp3.ctypes.data,
                                         sc.ctypes.data, ts.ctypes.data))
        return dict(bp1=bp1, bp2=bp2, bp3=bp3, mean1=sc[0], std1=sc[1], mean2=sc[2], std2=sc[3], ts=ts)

    def get_tuning(self) -> HellaTuning:
        t = HellaTuning()
        _chk(self.L.hella_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, t: HellaTuning):
        _chk(self.L.hella_set_tuning(self.h, C.byref(t)))

    def time_dedisp(self, t: HellaTuning | None = None, reps: int = 3) -> float:
        ms = C.c_float()
        _chk(self.L.hella_time_dedisp(self.h, None if t is None else C.byref(t), reps, C.byref(ms)))
        return ms.value

    def autotune(self, reps: int = 2):
        t, ms = HellaTuning(), C.c_float()
        _chk(self.L.hella_autotune(self.h, reps, C.byref(t), C.byref(ms)))
        return t, ms.value

    def flag_spec(self) -> np.ndarray:
        out = np.zeros(self.params.nchan, np.float32)
        _chk(self.L.hella_get_flag_spec(self.h, out.ctypes.data))
        return out


# ----------------------------------------------------------- batched search

class Batch:
    """All beams per launch (hella_batch_create ... hella_batch_destroy).
    dm_max: per-beam DM ceilings; killmask: [nbeam][nchan] (0 = dropped)."""

    def __init__(self, base: HellaParams, dm_max=None, killmask=None, widths_per_pass: int = 0,
                 use_graph: bool = True, dynamic: bool = False, member=None, inflight: int = 1,
                 bp_alpha: float = 0.1):
        self.L = lib()
        bp = batch_params(base, dm_max, killmask, widths_per_pass, use_graph, dynamic, member, inflight,
                          bp_alpha)
        self._keep = bp._keep
        h = _VP()
        _chk(self.L.hella_batch_create(C.byref(h), C.byref(bp)))
        self.h = h
        self.base = base
        self.nbeam = base.nbeam

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def submit(self, gulp, on_device=False):
        _chk(self.L.hella_batch_submit(self.h, _ptr(gulp), int(on_device)))

    def poll(self):
        """(candidates, counts, searched, latency_ms, device_ms) of the oldest submitted gulp."""
        cap = self.base.max_giants * self.nbeam
        out = np.zeros(cap, CAND_DTYPE)
        counts = np.zeros(self.nbeam, np.int32)
        searched = np.zeros(self.nbeam, np.int32)
        n, lat, dev = C.c_int(), C.c_float(), C.c_float()
        _chk(self.L.hella_batch_poll(self.h, out.ctypes.data, cap, C.byref(n), counts.ctypes.data,
                                     searched.ctypes.data, C.byref(lat), C.byref(dev)))
        return out[: n.value], counts, searched.astype(bool), lat.value, dev.value

    def set_beam(self, beam: int, member: bool, dm_max: float = 0.0, killmask=None):
        km = None if killmask is None else np.ascontiguousarray(killmask, dtype=np.int32)
        _chk(self.L.hella_batch_set_beam(self.h, beam, int(member), dm_max, None if km is None else km.ctypes.data))

    def flag_spec(self) -> np.ndarray:
        out = np.zeros(self.base.nchan, np.float32)
        _chk(self.L.hella_batch_get_flag_spec(self.h, out.ctypes.data))
        return out

    def bandpass(self, beam: int) -> np.ndarray:
        out = np.zeros(self.base.nchan, np.float32)
        _chk(self.L.hella_batch_get_bandpass(self.h, beam, out.ctypes.data))
        return out

    def info(self, beam: int) -> HellaInfo:
        i = HellaInfo()
        _chk(self.L.hella_batch_get_info(self.h, beam, C.byref(i)))
        return i

    def set_stream(self, stream: int):
        _chk(self.L.hella_batch_set_stream(self.h, stream))

    def process_gulp(self, gulp, on_device=False):
        """Returns (candidates, counts[nbeam], searched[nbeam])."""
        cap = self.base.max_giants * self.nbeam
        out = np.zeros(cap, CAND_DTYPE)
        counts = np.zeros(self.nbeam, np.int32)
        searched = np.zeros(self.nbeam, np.int32)
        n = C.c_int()
        _chk(self.L.hella_batch_process_gulp(self.h, _ptr(gulp), int(on_device), out.ctypes.data, cap,
                                             C.byref(n), counts.ctypes.data, searched.ctypes.data))
        return out[: n.value], counts, searched.astype(bool)

    def copy_dedisp(self, beam: int) -> np.ndarray:
        i = self.info(beam)
        out = np.empty((i.ndms, i.ntime_dd), np.float32)
        _chk(self.L.hella_batch_copy_dedisp(self.h, beam, out.ctypes.data))
        return out

    def get_tuning(self) -> HellaTuning:
        t = HellaTuning()
        _chk(self.L.hella_batch_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, t: HellaTuning):
        _chk(self.L.hella_batch_set_tuning(self.h, C.byref(t)))

    def time_dedisp(self, t: HellaTuning | None = None, reps: int = 3) -> float:
        ms = C.c_float()
        _chk(self.L.hella_batch_time_dedisp(self.h, None if t is None else C.byref(t), reps, C.byref(ms)))
        return ms.value

    def autotune(self, reps: int = 2):
        t, ms = HellaTuning(), C.c_float()
        _chk(self.L.hella_batch_autotune(self.h, reps, C.byref(t), C.byref(ms)))
        return t, ms.value

    def graph_kernels(self) -> int:
        n = C.c_int()
        _chk(self.L.hella_batch_graph_kernels(self.h, C.byref(n)))
        return n.value

    def last_gulp_ms(self) -> float:
        ms = C.c_float()
        _chk(self.L.hella_batch_last_gulp_ms(self.h, C.byref(ms)))
        return ms.value


def batch_params(base: HellaParams, dm_max=None, killmask=None, widths_per_pass: int = 0, use_graph: bool = True,
                 dynamic: bool = False, member=None, inflight: int = 1, bp_alpha: float = 0.1) -> BatchParams:
    bp = BatchParams()
    lib().hella_batch_params_default(C.byref(bp))
    bp.base = base
    keep = [None if dm_max is None else np.ascontiguousarray(dm_max, dtype=np.float32),
            None if killmask is None else np.ascontiguousarray(killmask, dtype=np.int32),
            None if member is None else np.ascontiguousarray(member, dtype=np.int32)]
    bp.dm_max = None if keep[0] is None else keep[0].ctypes.data
    bp.killmask = None if keep[1] is None else keep[1].ctypes.data
    bp.member = None if keep[2] is None else keep[2].ctypes.data
    bp.widths_per_pass = widths_per_pass
    bp.use_graph = int(use_graph)
    bp.dynamic = int(dynamic)
    bp.inflight = inflight
    bp.bp_alpha = bp_alpha
    bp._keep = keep
    return bp


def batch_bytes(base: HellaParams, **kw) -> int:
    """Device bytes a batch with these parameters holds (hella_batch_bytes)."""
    bp = batch_params(base, **kw)
    n = C.c_size_t()
    _chk(lib().hella_batch_bytes(C.byref(bp), C.byref(n)))
    return n.value


# --------------------------------------------------------- candidate refinement

class Refine:
    """Differentiable candidate refinement (hella_refine_*).  Arguments are
    CUDA tensors: cutouts f32 [n][nchan][nsamp], dm_ref f32 [n], theta f32
    [n][5] = (dm, t0, width_ms, amp, index)."""

    def __init__(self, ncut: int, nchan: int, nsamp: int, tsamp: float, f0_mhz: float, df_mhz: float,
                 device: int = 0, stream: int | None = None):
        self.L = lib()
        p = RefineParams(ncut, nchan, nsamp, tsamp, f0_mhz, df_mhz, device)
        h = _VP()
        _chk(self.L.hella_refine_create(C.byref(h), C.byref(p)))
        self.h, self.p = h, p
        if stream is not None:
            _chk(self.L.hella_refine_set_stream(self.h, stream))

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_refine_destroy(self.h)
            self.h = None

    __del__ = close

    def set_stream(self, stream: int):
        _chk(self.L.hella_refine_set_stream(self.h, stream))

    def delay_table(self) -> np.ndarray:
        out = np.zeros(self.p.nchan, np.float32)
        _chk(self.L.hella_refine_delay_table(self.h, out.ctypes.data))
        return out

    def forward(self, cut, dm_ref, theta, chi2):
        _chk(self.L.hella_refine_forward(self.h, theta.shape[0], _ptr(cut), _ptr(dm_ref), _ptr(theta), _ptr(chi2)))

    def adjoint(self, cut, dm_ref, theta, gchi2, gtheta):
        _chk(self.L.hella_refine_adjoint(self.h, theta.shape[0], _ptr(cut), _ptr(dm_ref), _ptr(theta), _ptr(gchi2),
                                         _ptr(gtheta)))

    def fit(self, cut, dm_ref, theta, steps: int, lr, chi2=None):
        lr = np.ascontiguousarray(lr, dtype=np.float32)
        _chk(self.L.hella_refine_fit(self.h, theta.shape[0], _ptr(cut), _ptr(dm_ref), _ptr(theta), steps,
                                     lr.ctypes.data, _ptr(chi2)))


# ------------------------------------------------------------------- I/O

class Filterbank:
    """SIGPROC filterbank reader (hella_fil_*)."""

    def __init__(self, path: str, expect_nchan: int = 0):
        self.L = lib()
        h, hdr = _VP(), FilHeader()
        _chk(self.L.hella_fil_open(C.byref(h), str(path).encode(), expect_nchan, C.byref(hdr)))
        self.h, self.header = h, hdr

    def read(self, nsamp: int) -> np.ndarray:
        out = np.empty((nsamp, self.header.nchans), np.uint8)
        got = C.c_int()
        _chk(self.L.hella_fil_read(self.h, out.ctypes.data, nsamp, C.byref(got)))
        return out[: got.value]

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_fil_close(self.h)
            self.h = None

    __del__ = close


def _cands_arg(c):
    c = np.ascontiguousarray(c, CAND_DTYPE)
    return c, (c.ctypes.data if len(c) else None)


def cands_format(cands, samp0: int, dms, time_resolution: float = 1.0e-3) -> str:
    c, cp = _cands_arg(cands)
    d = np.ascontiguousarray(dms, np.float32)
    buf = C.create_string_buffer(96 * len(c) + 64)
    n = C.c_size_t()
    _chk(lib().hella_cands_format(cp, len(c), samp0, d.ctypes.data, len(d), time_resolution, buf, len(buf),
                                  C.byref(n)))
    return buf.raw[: n.value].decode()


def cands_append(path: str, cands, samp0: int, dms, time_resolution: float = 1.0e-3):
    c, cp = _cands_arg(cands)
    d = np.ascontiguousarray(dms, np.float32)
    _chk(lib().hella_cands_append(str(path).encode(), cp, len(c), samp0, d.ctypes.data, len(d), time_resolution))


def cands_coincidencer(gulp_number: int, cands, samp0: int, dms, time_resolution: float = 1.0e-3,
                       utc_start=None, picoseconds=None, tsamp=None) -> str:
    c, cp = _cands_arg(cands)
    d = np.ascontiguousarray(dms, np.float32)
    buf = C.create_string_buffer(96 * len(c) + 256)
    n = C.c_size_t()
    enc = lambda v: None if v is None else str(v).encode()
    _chk(lib().hella_cands_coincidencer(gulp_number, enc(utc_start), enc(picoseconds), enc(tsamp), cp, len(c),
                                        samp0, d.ctypes.data, len(d), time_resolution, buf, len(buf), C.byref(n)))
    return buf.raw[: n.value].decode()


def cands_send(host: str, port: int, message, timeout_ms: int = 2000):
    """Sends one message (str or bytes) to host:port over TCP (hella_cands_send)."""
    data = message.encode() if isinstance(message, str) else bytes(message)
    _chk(lib().hella_cands_send(host.encode(), port, data, len(data), timeout_ms))


def cluster(cands, dsamp: int, ddm: int, dwidth: int):
    """(representatives, labels) of friends-of-friends clusters (hella_cluster)."""
    c, cp = _cands_arg(cands)
    out = np.zeros(max(1, len(c)), CAND_DTYPE)
    labels = np.zeros(max(1, len(c)), np.int32)
    n = C.c_int()
    _chk(lib().hella_cluster(cp, len(c), dsamp, ddm, dwidth, out.ctypes.data, C.byref(n), labels.ctypes.data))
    return out[: n.value], labels[: len(c)]


class FlagStats:
    """Per-channel flag counts over searched gulps (hella_flagstats_*)."""

    def __init__(self, nchan: int, ntime: int):
        self.L = lib()
        h = _VP()
        _chk(self.L.hella_flagstats_create(C.byref(h), nchan, ntime))
        self.h, self.nchan = h, nchan

    def update(self, cumulative):
        a = np.ascontiguousarray(cumulative, np.float32)
        _chk(self.L.hella_flagstats_update(self.h, a.ctypes.data))

    def counts(self) -> np.ndarray:
        out = np.zeros(self.nchan, np.int64)
        _chk(self.L.hella_flagstats_counts(self.h, out.ctypes.data))
        return out

    def append(self, path: str):
        _chk(self.L.hella_flagstats_append(self.h, str(path).encode()))

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_flagstats_destroy(self.h)
            self.h = None

    __del__ = close


class Ring:
    """In-process header + data-block ring (hella_ring_*)."""

    def __init__(self, block_bytes: int, nblocks: int, pinned: bool = False):
        self.L = lib()
        h = _VP()
        _chk(self.L.hella_ring_create(C.byref(h), block_bytes, nblocks, int(pinned)))
        self.h, self.block_bytes = h, block_bytes

    def close(self):
        if getattr(self, "h", None):
            self.L.hella_ring_destroy(self.h)
            self.h = None

    __del__ = close

    def write_header(self, text: str):
        b = text.encode()
        _chk(self.L.hella_ring_write_header(self.h, b, len(b)))

    def read_header(self, timeout_ms: int = 1000) -> str:
        buf = C.create_string_buffer(65536)
        n = C.c_size_t()
        _chk(self.L.hella_ring_read_header(self.h, buf, len(buf), C.byref(n), timeout_ms))
        return buf.raw[: n.value].decode()

    def write(self, data: bytes, timeout_ms: int = 1000):
        p = _VP()
        _chk(self.L.hella_ring_open_write(self.h, C.byref(p), timeout_ms))
        C.memmove(p, data, len(data))
        _chk(self.L.hella_ring_mark_filled(self.h, len(data)))

    def end(self):
        _chk(self.L.hella_ring_end(self.h))

    def open_read(self, timeout_ms: int = 1000):
        """(address, nbytes) of the next filled block, left in place until
        mark_cleared(); nbytes == 0 at the end of the data."""
        p, n = _VP(), C.c_size_t()
        _chk(self.L.hella_ring_open_read(self.h, C.byref(p), C.byref(n), timeout_ms))
        return (p.value or 0), n.value

    def mark_cleared(self):
        _chk(self.L.hella_ring_mark_cleared(self.h))

    def read(self, timeout_ms: int = 1000):
        """bytes of the next block, or None at the end of the data."""
        p, n = _VP(), C.c_size_t()
        _chk(self.L.hella_ring_open_read(self.h, C.byref(p), C.byref(n), timeout_ms))
        if n.value == 0:
            return None
        data = C.string_at(p, n.value)
        _chk(self.L.hella_ring_mark_cleared(self.h))
        return data


def header_get(header: str, key: str):
    b = header.encode()
    out = C.create_string_buffer(4096)
    rc = lib().hella_header_get(b, len(b), key.encode(), out, len(out))
    return out.value.decode() if rc == 0 else None
