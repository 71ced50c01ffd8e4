// plan.cpp -- the hdd_ plan/execute API (include/hella_dedisp.h).
//
// Host side of dedispersion: DM list, delay table, killmask, and the
// execute calls that casm-hella makes through dedisp
// (src/apps/casm_hella_refactored.cu:205-210, src/hella/src/dedisperse.cpp:
// 17-48).  The device work is in dedisp.cu.
#include "hella_dedisp.h"
#include "hg_internal.h"
#include "hg_plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace hg {

// DM trials from a smearing tolerance (Cordes & McLaughlin 2003; the rule
// of brute-force dedispersion codes, Barsdell et al. 2012).  With ts the
// sample time, ti the pulse width, a = 8.3 us |df| / f^3 the in-channel
// smearing per unit DM at the band centre f (GHz) and b = a*nchan/4 the
// band smearing per unit DM error, the next trial D' satisfies
//   ts^2 + ti^2 + a^2 D'^2 + b^2 (D' - D)^2 = tol^2 (ts^2 + ti^2 + a^2 D^2),
// whose larger root is taken.  Trials stop at the first one >= dm_end.
std::vector<float> generate_dm_list(double dm_start, double dm_end, double ti_us,
                                    double tol, int nchan, double dt_s, double f0,
                                    double df) {
  const double ts = dt_s * 1e6;
  const double adf = std::fabs(df);
  const double f = (f0 - (nchan * 0.5 - 0.5) * adf) * 1e-3;
  const double tol2 = tol * tol;
  const double a = 8.3 * adf / (f * f * f);
  const double a2 = a * a;
  const double b2 = a2 * (double)nchan * (double)nchan / 16.0;
  const double c = (ts * ts + ti_us * ti_us) * (tol2 - 1.0);
  std::vector<float> out;
  double dm = dm_start;
  out.push_back((float)dm);
  while (dm < dm_end && out.size() < (1u << 22)) {
    const double d2 = dm * dm;
    const double k = c + tol2 * a2 * d2;
    dm = (b2 * dm + std::sqrt(-a2 * b2 * d2 + (a2 + b2) * k)) / (a2 + b2);
    out.push_back((float)dm);
  }
  return out;
}

// Samples of delay per unit DM, relative to channel 0 (frequency f0):
// 4.148808e3 s MHz^2 (1/f_c^2 - 1/f0^2) / dt with f_c = f0 - c |df|.
std::vector<float> delay_table(int nchan, double dt_s, double f0, double df) {
  std::vector<float> t(nchan);
  const double adf = std::fabs(df);
  for (int c = 0; c < nchan; ++c) {
    const double fc = f0 - c * adf;
    t[c] = (float)(4.148808e3 / dt_s * (1.0 / (fc * fc) - 1.0 / (f0 * f0)));
  }
  return t;
}

// delay(c, d) = (int)(DM_d * table[c] + 0.5f), each operation in fp32.
std::vector<int> dm_delays(const std::vector<float> &dms, const std::vector<float> &table) {
  const size_t nchan = table.size();
  std::vector<int> d(dms.size() * nchan);
  for (size_t i = 0; i < dms.size(); ++i)
    for (size_t c = 0; c < nchan; ++c) {
      float p = dms[i] * table[c];
      p = p + 0.5f;
      d[i * nchan + c] = (int)p;
    }
  return d;
}

}  // namespace hg

struct hdd_plan_struct {
  int device = 0;
  cudaStream_t stream = nullptr;
  int nchans = 0;
  float dt = 0, f0 = 0, df = 0;
  std::vector<float> table, dms;
  std::vector<int> delays, chans;
  std::vector<hdd_bool> killmask;
  int max_delay = 0;
  // dedispersion tile tables of the last DM range used, host and device
  hg::DedispTables tab;
  int tab_first = -1, tab_count = -1, tab_dpt = -1, tab_cc = -1;
  bool tab_on_device = false;
  int *d_err = nullptr;  // dedispersion status word
  int4 *d_meta = nullptr;
  int *d_off = nullptr;
  size_t meta_cap = 0, off_cap = 0;
  uint8_t *d_in = nullptr, *d_plain = nullptr, *d_out = nullptr;
  uint32_t *d_packed = nullptr;
  size_t in_cap = 0, plain_cap = 0, out_cap = 0, packed_cap = 0;
  // add-mode-4 tables of the last DM range used, host and device
  hg::SubTables sub;
  int sub_first = -1, sub_count = -1;
  bool sub_on_device = false;
  int4 *d_smeta = nullptr;
  int2 *d_sindex = nullptr;
  int *d_spool = nullptr;
  size_t smeta_cap = 0, sindex_cap = 0, spool_cap = 0;
  // add-mode-5 tables of the last DM range and shape used, host and device, and the rows
  hg::PairTables pair;
  int pair_rows = 0;  // hdd_set_pair_rows: channels a group (2 or 4) of the execute calls' rows; 0: off
  int pair_first = -1, pair_count = -1, pair_cc = -1, pair_ntt = -1, pair_g = -1;
  bool pair_on_device = false;
  int4 *d_prinfo = nullptr, *d_prinfo2 = nullptr, *d_prec = nullptr;
  long long *d_proff = nullptr;
  int *d_prwords = nullptr, *d_prtile = nullptr, *d_pprow = nullptr, *d_ptile = nullptr;
  int2 *d_pprange = nullptr;
  uint32_t *d_prows = nullptr;
  size_t prinfo_cap = 0, prinfo2_cap = 0, prtile_cap = 0, prec_cap = 0, proff_cap = 0, prwords_cap = 0, pprow_cap = 0, ptile_cap = 0,
         pprange_cap = 0, prows_cap = 0;
};

namespace {

thread_local int t_device = 0;

void invalidate_tables(hdd_plan p) {
  p->tab_first = p->tab_count = p->tab_dpt = p->tab_cc = -1;
  p->tab_on_device = false;
  p->sub_first = p->sub_count = -1;
  p->sub_on_device = false;
  p->pair_first = p->pair_count = p->pair_cc = p->pair_ntt = p->pair_g = -1;
  p->pair_on_device = false;
}

// Delays of the plan's DM list; max_delay is the largest of them (the last
// trial's lowest channel for an ascending list, any trial for another order).
hdd_error refresh_delays(hdd_plan p) {
  invalidate_tables(p);
  try {
    p->delays = hg::dm_delays(p->dms, p->table);
  } catch (const std::bad_alloc &) {
    p->dms.clear();
    p->delays.clear();
    p->max_delay = 0;
    return HDD_MEM_ALLOC_FAILED;
  }
  p->max_delay = p->delays.empty() ? 0 : *std::max_element(p->delays.begin(), p->delays.end());
  return HDD_NO_ERROR;
}

// A trial the kernels can serve: finite, not negative, and a delay that
// stays far inside int (the delay table grows with channel index).
bool dm_ok(hdd_plan p, float dm) {
  if (!(dm >= 0.f) || !(dm < 3.0e38f)) return false;
  return (double)dm * p->table[p->nchans - 1] + 0.5 < (double)(1 << 30);
}

void rebuild_chans(hdd_plan p) {
  p->chans.clear();
  for (int c = 0; c < p->nchans; ++c)
    if (p->killmask[c]) p->chans.push_back(c);
  invalidate_tables(p);
}

hdd_error grow(void **ptr, size_t *cap, size_t need) {
  if (*cap >= need) return HDD_NO_ERROR;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  if (cudaMalloc(ptr, need) != cudaSuccess) {
    cudaGetLastError();
    return HDD_MEM_ALLOC_FAILED;
  }
  *cap = need;
  return HDD_NO_ERROR;
}

}  // namespace

namespace hg {

const DedispTables &plan_host_tables(hdd_plan p, int first, int count, int dpt, int cc) {
  if (p->tab_first != first || p->tab_count != count || p->tab_dpt != dpt || p->tab_cc != cc) {
    p->tab = dedisp_tables(p->delays.data(), p->nchans, p->chans.data(), (int)p->chans.size(), first,
                           count, dpt, cc);
    p->tab_first = first;
    p->tab_count = count;
    p->tab_dpt = dpt;
    p->tab_cc = cc;
    p->tab_on_device = false;
  }
  return p->tab;
}

hdd_error plan_device_tables(hdd_plan p, int first, int count, DeviceTables *out, int dpt, int cc) {
  const DedispTables &t = plan_host_tables(p, first, count, dpt, cc);
  if (!p->tab_on_device) {
    const size_t mb = std::max<size_t>(t.meta.size(), 1) * sizeof(int4);
    const size_t ob = std::max<size_t>(t.off.size(), 1) * sizeof(int);
    hdd_error e;
    if ((e = grow((void **)&p->d_meta, &p->meta_cap, mb)) != HDD_NO_ERROR) return e;
    if ((e = grow((void **)&p->d_off, &p->off_cap, ob)) != HDD_NO_ERROR) return e;
    if (!t.meta.empty() &&
        (cudaMemcpy(p->d_meta, t.meta.data(), t.meta.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess ||
         cudaMemcpy(p->d_off, t.off.data(), t.off.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess))
      return HDD_MEM_COPY_FAILED;
    p->tab_on_device = true;
  }
  out->meta = p->d_meta;
  out->off = p->d_off;
  out->dpt = t.dpt;
  out->max_spread = t.max_spread;
  out->nact = (int)p->chans.size();
  out->cc = cc;
  return HDD_NO_ERROR;
}

hdd_error plan_sub_tables(hdd_plan p, int first, int count, SubDeviceTables *out) {
  if (p->sub_first != first || p->sub_count != count) {
    try {
      p->sub = dedisp_sub_tables(p->delays.data(), p->nchans, p->chans.data(), (int)p->chans.size(), first, count);
    } catch (const std::bad_alloc &) {
      p->sub_first = p->sub_count = -1;
      return HDD_MEM_ALLOC_FAILED;
    }
    p->sub_first = first;
    p->sub_count = count;
    p->sub_on_device = false;
  }
  const SubTables &t = p->sub;
  if (!p->sub_on_device) {
    hdd_error e;
    if ((e = grow((void **)&p->d_smeta, &p->smeta_cap, std::max<size_t>(t.meta.size(), 1) * sizeof(int4))) !=
            HDD_NO_ERROR ||
        (e = grow((void **)&p->d_sindex, &p->sindex_cap, std::max<size_t>(t.index.size(), 1) * sizeof(int2))) !=
            HDD_NO_ERROR ||
        (e = grow((void **)&p->d_spool, &p->spool_cap, std::max<size_t>(t.pool.size(), 1) * sizeof(int))) !=
            HDD_NO_ERROR)
      return e;
    if (!t.meta.empty() &&
        (cudaMemcpy(p->d_smeta, t.meta.data(), t.meta.size() * sizeof(int4), cudaMemcpyHostToDevice) !=
             cudaSuccess ||
         cudaMemcpy(p->d_sindex, t.index.data(), t.index.size() * sizeof(int2), cudaMemcpyHostToDevice) !=
             cudaSuccess ||
         cudaMemcpy(p->d_spool, t.pool.data(), t.pool.size() * sizeof(int), cudaMemcpyHostToDevice) !=
             cudaSuccess))
      return HDD_MEM_COPY_FAILED;
    p->sub_on_device = true;
  }
  out->meta = p->d_smeta;
  out->index = p->d_sindex;
  out->pool = p->d_spool;
  out->max_spread = t.max_spread;
  out->max_words = t.max_words;
  out->max_rec = t.max_rec;
  out->nact = (int)p->chans.size();
  return HDD_NO_ERROR;
}

// Host pair tables of the range and shape, built when they differ from the cached ones.
hdd_error pair_host_tables(hdd_plan p, int first, int count, int cc, int ntt, int g) {
  if (p->pair_first == first && p->pair_count == count && p->pair_cc == cc && p->pair_ntt == ntt &&
      p->pair_g == g)
    return HDD_NO_ERROR;
  try {
    p->pair = dedisp_pair_tables(p->delays.data(), p->nchans, p->chans.data(), (int)p->chans.size(), first, count,
                                 cc, ntt, g);
  } catch (const std::bad_alloc &) {
    p->pair_first = p->pair_count = p->pair_cc = p->pair_ntt = p->pair_g = -1;
    return HDD_MEM_ALLOC_FAILED;
  }
  p->pair_first = first;
  p->pair_count = count;
  p->pair_cc = cc;
  p->pair_ntt = ntt;
  p->pair_g = g;
  p->pair_on_device = false;
  return HDD_NO_ERROR;
}

namespace {

template <class T>
size_t vbytes(const std::vector<T> &v) {
  return std::max<size_t>(v.size(), 1) * sizeof(T);
}

}  // namespace

hdd_error plan_pair_bytes(hdd_plan p, int first, int count, int cc, int ntt, int g, size_t *bytes) {
  const hdd_error e = pair_host_tables(p, first, count, cc, ntt, g);
  if (e != HDD_NO_ERROR) return e;
  const PairTables &t = p->pair;
  *bytes = vbytes(t.rinfo) + vbytes(t.rinfo2) + vbytes(t.roff) + vbytes(t.rwords) + vbytes(t.rtile) + vbytes(t.prow) + vbytes(t.prange) +
           vbytes(t.rec) + vbytes(t.tile_st) + std::max<size_t>((size_t)t.words, 4) * 4;
  return HDD_NO_ERROR;
}

hdd_error plan_pair_tables(hdd_plan p, int first, int count, int cc, int ntt, int g, PairDeviceTables *out,
                           bool rows) {
  hdd_error e = pair_host_tables(p, first, count, cc, ntt, g);
  if (e != HDD_NO_ERROR) return e;
  const PairTables &t = p->pair;
  if (!p->pair_on_device) {
    auto up = [&](void **d, size_t *cap, const void *src, size_t n) -> hdd_error {
      hdd_error r = grow(d, cap, std::max<size_t>(n, 16));
      if (r != HDD_NO_ERROR) return r;
      if (n && cudaMemcpy(*d, src, n, cudaMemcpyHostToDevice) != cudaSuccess) return HDD_MEM_COPY_FAILED;
      return HDD_NO_ERROR;
    };
    if ((e = up((void **)&p->d_prinfo, &p->prinfo_cap, t.rinfo.data(), t.rinfo.size() * sizeof(int4))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_prinfo2, &p->prinfo2_cap, t.rinfo2.data(), t.rinfo2.size() * sizeof(int4))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_proff, &p->proff_cap, t.roff.data(), t.roff.size() * sizeof(long long))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_prwords, &p->prwords_cap, t.rwords.data(), t.rwords.size() * sizeof(int))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_prtile, &p->prtile_cap, t.rtile.data(), t.rtile.size() * sizeof(int))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_pprow, &p->pprow_cap, t.prow.data(), t.prow.size() * sizeof(int))) != HDD_NO_ERROR ||
        (e = up((void **)&p->d_pprange, &p->pprange_cap, t.prange.data(), t.prange.size() * sizeof(int2))) !=
            HDD_NO_ERROR ||
        (e = up((void **)&p->d_prec, &p->prec_cap, t.rec.data(), t.rec.size() * sizeof(int4))) != HDD_NO_ERROR ||
        (e = up((void **)&p->d_ptile, &p->ptile_cap, t.tile_st.data(), t.tile_st.size() * sizeof(int))) !=
            HDD_NO_ERROR)
      return e;
    p->pair_on_device = true;
  }
  if (rows && (e = grow((void **)&p->d_prows, &p->prows_cap, std::max<size_t>((size_t)t.words, 4) * 4)) !=
                  HDD_NO_ERROR)
    return e;
  out->rinfo = p->d_prinfo;
  out->rinfo2 = p->d_prinfo2;
  out->roff = p->d_proff;
  out->rwords = p->d_prwords;
  out->rtile = p->d_prtile;
  out->prow = p->d_pprow;
  out->prange = p->d_pprange;
  out->rec = p->d_prec;
  out->tile_st = p->d_ptile;
  out->rows = rows ? p->d_prows : nullptr;
  out->words = t.words;
  out->npair = t.npair;
  out->span = t.max_span;
  out->stage = t.max_stage;
  out->nact = (int)p->chans.size();
  out->cc = t.cc;
  out->g = t.g;
  out->npos = t.npos;
  return HDD_NO_ERROR;
}

void plan_pair_release(hdd_plan p) {
  if (!p || !(p->d_prinfo || p->d_prows)) return;
  cudaSetDevice(p->device);
  void **bufs[] = {(void **)&p->d_prinfo, (void **)&p->d_prinfo2, (void **)&p->d_proff, (void **)&p->d_prwords,
                   (void **)&p->d_prtile, (void **)&p->d_pprow, (void **)&p->d_pprange, (void **)&p->d_prec,
                   (void **)&p->d_ptile, (void **)&p->d_prows};
  size_t *caps[] = {&p->prinfo_cap, &p->prinfo2_cap, &p->proff_cap, &p->prwords_cap, &p->prtile_cap,
                    &p->pprow_cap, &p->pprange_cap, &p->prec_cap, &p->ptile_cap, &p->prows_cap};
  for (int i = 0; i < 10; ++i) {
    cudaFree(*bufs[i]);
    *bufs[i] = nullptr;
    *caps[i] = 0;
  }
  p->pair_on_device = false;
}

hdd_error plan_pair_row_ends(hdd_plan p, int count, int *ends) {
  if (p->pair_first != 0 || count > p->pair_count) return HDD_UNKNOWN_ERROR;
  pair_row_ends(p->pair, count, ends);
  return HDD_NO_ERROR;
}

void use_pair_tables(DedispArgs *a, const PairDeviceTables &t) {
  a->dpt = kPairDPT;
  a->mode = t.g == 4 ? 6 : 5;
  a->cc = t.cc;
  a->nact = t.nact;
  a->pair_g = t.g;
  a->pair_lanecap = pair_lanecap(t.g);
  a->pair_rinfo = t.rinfo;
  a->pair_rinfo2 = t.rinfo2;
  a->pair_roff = t.roff;
  a->pair_rwords = t.rwords;
  a->pair_rtile = t.rtile;
  a->pair_prow = t.prow;
  a->pair_prange = t.prange;
  a->pair_rec = t.rec;
  a->pair_tile_st = t.tile_st;
  a->pair_rows = t.rows;
  a->pair_rows_stride = t.words;
  a->pair_npair = t.npair;
  a->pair_span = t.span;
  a->pair_stage = t.stage;
  a->pair_npos = t.npos;
}

void use_sub_tables(DedispArgs *a, const SubDeviceTables &t) {
  a->dpt = kSubDPT;
  a->mode = 4;
  a->nact = t.nact;
  a->max_spread = t.max_spread;
  a->tile_meta = t.meta;
  a->tile_off = nullptr;
  a->sub_index = t.index;
  a->sub_pool = t.pool;
  a->sub_words = t.max_words;
  a->sub_rec = t.max_rec;
}

DedispArgs single_beam_args(const DeviceTables &tb, const uint32_t *packed, long R, long win0,
                            int dm_first, int dm_count, int nout, float *out, long out_stride,
                            int *err) {
  DedispArgs a{};
  a.beams = nullptr;
  a.one.packed = packed;
  a.one.out = out;
  a.one.win0 = win0;
  a.one.dm_count = dm_count;
  a.one.item0 = 0;
  a.nbeam = 1;
  a.ntt = dedisp_time_tiles(nout);
  a.nitems = dedisp_items(dm_count, tb.dpt, a.ntt);
  a.group = kDedispGroup;
  a.R = R;
  a.nact = tb.nact;
  a.dm_first = dm_first;
  a.nout = nout;
  a.out_stride = out_stride;
  a.dpt = tb.dpt;
  a.cc = tb.cc;
  a.max_spread = tb.max_spread;
  a.tile_meta = tb.meta;
  a.tile_off = tb.off;
  a.err = err;
  a.unit = 1;
  return a;
}

PlanView plan_view(hdd_plan p) {
  PlanView v{};
  v.device = p->device;
  v.stream = p->stream;
  v.nchans = p->nchans;
  v.ndms = (int)p->dms.size();
  v.max_delay = p->max_delay;
  v.delays = p->delays.empty() ? nullptr : p->delays.data();
  v.chans = p->chans.empty() ? nullptr : p->chans.data();
  v.nact = (int)p->chans.size();
  return v;
}

}  // namespace hg

extern "C" {

hdd_error hdd_create_plan(hdd_plan *plan, hdd_size nchans, hdd_float dt, hdd_float f0,
                          hdd_float df) {
  if (!plan) return HDD_INVALID_POINTER;
  *plan = nullptr;
  if (nchans == 0 || nchans > HDD_MAX_NCHANS) return HDD_NCHANS_EXCEEDS_LIMIT;
  if (!(dt > 0) || !(f0 > 0) || !(df != 0)) return HDD_UNKNOWN_ERROR;
  hdd_plan p = new (std::nothrow) hdd_plan_struct;
  if (!p) return HDD_MEM_ALLOC_FAILED;
  p->device = t_device;
  p->nchans = (int)nchans;
  p->dt = dt;
  p->f0 = f0;
  p->df = df;
  p->table = hg::delay_table(p->nchans, dt, f0, df);
  p->killmask.assign(p->nchans, 1);
  rebuild_chans(p);
  *plan = p;
  return HDD_NO_ERROR;
}

void hdd_destroy_plan(hdd_plan p) {
  if (!p) return;
  cudaSetDevice(p->device);
  cudaFree(p->d_meta);
  cudaFree(p->d_off);
  cudaFree(p->d_err);
  cudaFree(p->d_in);
  cudaFree(p->d_plain);
  cudaFree(p->d_packed);
  cudaFree(p->d_out);
  cudaFree(p->d_smeta);
  cudaFree(p->d_sindex);
  cudaFree(p->d_spool);
  cudaFree(p->d_prinfo);
  cudaFree(p->d_prinfo2);
  cudaFree(p->d_proff);
  cudaFree(p->d_prwords);
  cudaFree(p->d_prtile);
  cudaFree(p->d_pprow);
  cudaFree(p->d_pprange);
  cudaFree(p->d_prec);
  cudaFree(p->d_ptile);
  cudaFree(p->d_prows);
  delete p;
}

hdd_error hdd_set_device(int device_idx) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return HDD_INVALID_DEVICE_INDEX;
  }
  if (device_idx < 0 || device_idx >= n) return HDD_INVALID_DEVICE_INDEX;
  if (cudaSetDevice(device_idx) != cudaSuccess) return HDD_INVALID_DEVICE_INDEX;
  t_device = device_idx;
  return HDD_NO_ERROR;
}

hdd_error hdd_set_pair_rows(hdd_plan p, int channels) {
  if (!p) return HDD_INVALID_PLAN;
  if (channels != 0 && channels != 1 && channels != 2 && channels != 4) return HDD_UNKNOWN_ERROR;
  p->pair_rows = channels == 1 ? 2 : channels;
  if (!p->pair_rows) hg::plan_pair_release(p);
  return HDD_NO_ERROR;
}

hdd_error hdd_get_pair_tables(hdd_plan p, hdd_size first, hdd_size count, int channels, int stage_groups,
                              int time_tiles, hdd_pair_tables_view *out) {
  if (!p) return HDD_INVALID_PLAN;
  if (!out) return HDD_INVALID_POINTER;
  if (p->dms.empty()) return HDD_NO_DM_LIST_SET;
  if ((channels != 2 && channels != 4) || (stage_groups != 4 && stage_groups != 8) || time_tiles < 1 ||
      count == 0 || first + count > p->dms.size() || p->chans.empty())
    return HDD_UNKNOWN_ERROR;
  const hdd_error e = hg::pair_host_tables(p, (int)first, (int)count, stage_groups, time_tiles, channels);
  if (e != HDD_NO_ERROR) return e;
  const hg::PairTables &t = p->pair;
  out->channels = t.g;
  out->stage_groups = t.cc;
  out->time_tiles = t.ntt;
  out->ntiles = t.ntiles;
  out->ngroups = t.npair;
  out->nrows = t.nrows;
  out->rec_ints = hg::pair_rec_int4(t.cc) * 4;
  out->nrec = (int)(t.rec.size() / hg::pair_rec_int4(t.cc));
  out->max_stage_bytes = t.max_stage;
  out->max_span = t.max_span;
  out->npos = t.npos;
  out->words = t.words;
  out->rinfo = reinterpret_cast<const int *>(t.rinfo.data());
  out->rinfo2 = reinterpret_cast<const int *>(t.rinfo2.data());
  out->roff = t.roff.data();
  out->rwords = t.rwords.data();
  out->rtile = t.rtile.data();
  out->prow = t.prow.data();
  out->prange = reinterpret_cast<const int *>(t.prange.data());
  out->rec = reinterpret_cast<const int *>(t.rec.data());
  out->tile_st = t.tile_st.data();
  return HDD_NO_ERROR;
}

hdd_error hdd_set_stream(hdd_plan p, void *stream) {
  if (!p) return HDD_INVALID_PLAN;
  p->stream = (cudaStream_t)stream;
  return HDD_NO_ERROR;
}

hdd_error hdd_set_dm_list(hdd_plan p, const hdd_float *dm_list, hdd_size count) {
  if (!p) return HDD_INVALID_PLAN;
  if (!dm_list) return HDD_INVALID_POINTER;
  // any order; every trial finite, >= 0 and within the delay range
  for (hdd_size i = 0; i < count; ++i)
    if (!dm_ok(p, dm_list[i])) return HDD_UNKNOWN_ERROR;
  if (count > ((size_t)1 << 31) / (size_t)p->nchans) return HDD_MEM_ALLOC_FAILED;  // delay table
  try {
    p->dms.assign(dm_list, dm_list + count);
  } catch (const std::bad_alloc &) {
    return HDD_MEM_ALLOC_FAILED;
  }
  return refresh_delays(p);
}

hdd_error hdd_generate_dm_list(hdd_plan p, hdd_float dm_start, hdd_float dm_end, hdd_float ti,
                               hdd_float tol) {
  if (!p) return HDD_INVALID_PLAN;
  // dm_end below dm_start gives the single trial dm_start; tol <= 1 would
  // never advance
  if (!dm_ok(p, dm_start) || !std::isfinite(dm_end) || !std::isfinite(ti) || !(tol > 1.f) ||
      !std::isfinite(tol))
    return HDD_UNKNOWN_ERROR;
  std::vector<float> dms;
  try {
    dms = hg::generate_dm_list(dm_start, dm_end, ti, tol, p->nchans, p->dt, p->f0, p->df);
  } catch (const std::bad_alloc &) {
    return HDD_MEM_ALLOC_FAILED;
  }
  // the list ends at the first trial >= dm_end, which may pass the range
  if (!dm_ok(p, dms.back())) return HDD_UNKNOWN_ERROR;
  if (dms.size() > ((size_t)1 << 31) / (size_t)p->nchans) return HDD_MEM_ALLOC_FAILED;
  p->dms.swap(dms);
  return refresh_delays(p);
}

hdd_error hdd_set_killmask(hdd_plan p, const hdd_bool *killmask) {
  if (!p) return HDD_INVALID_PLAN;
  if (killmask)
    p->killmask.assign(killmask, killmask + p->nchans);
  else
    p->killmask.assign(p->nchans, 1);
  rebuild_chans(p);
  return HDD_NO_ERROR;
}

hdd_size hdd_get_max_delay(const hdd_plan p) { return p ? (hdd_size)p->max_delay : 0; }
hdd_size hdd_get_dm_delay(const hdd_plan p, int trial) {
  if (!p || trial < 0 || trial >= (int)p->dms.size()) return 0;
  return (hdd_size)p->delays[(size_t)trial * p->nchans + p->nchans - 1];
}
hdd_size hdd_get_channel_count(const hdd_plan p) { return p ? (hdd_size)p->nchans : 0; }
hdd_size hdd_get_dm_count(const hdd_plan p) { return p ? (hdd_size)p->dms.size() : 0; }
const hdd_float *hdd_get_dm_list(const hdd_plan p) {
  return (p && !p->dms.empty()) ? p->dms.data() : nullptr;
}
const hdd_bool *hdd_get_killmask(const hdd_plan p) { return p ? p->killmask.data() : nullptr; }
hdd_float hdd_get_dt(const hdd_plan p) { return p ? p->dt : 0.f; }
hdd_float hdd_get_df(const hdd_plan p) { return p ? p->df : 0.f; }
hdd_float hdd_get_f0(const hdd_plan p) { return p ? p->f0 : 0.f; }
const int *hdd_get_delay_table(const hdd_plan p) {
  return (p && !p->delays.empty()) ? p->delays.data() : nullptr;
}

hdd_error hdd_execute_guru(hdd_plan p, hdd_size nsamps, const hdd_byte *in, hdd_size in_nbits,
                           hdd_size in_stride, hdd_byte *out, hdd_size out_nbits,
                           hdd_size out_stride, hdd_size first_dm_idx, hdd_size dm_count,
                           unsigned flags) {
  if (!p) return HDD_INVALID_PLAN;
  if (!in || !out) return HDD_INVALID_POINTER;
  if (p->dms.empty()) return HDD_NO_DM_LIST_SET;
  if ((flags & HDD_HOST_POINTERS) && (flags & HDD_DEVICE_POINTERS))
    return HDD_INVALID_FLAG_COMBINATION;
  if ((flags & HDD_WAIT) && (flags & HDD_ASYNC)) return HDD_INVALID_FLAG_COMBINATION;
  if (in_nbits != 8) return HDD_UNSUPPORTED_IN_NBITS;
  if (out_nbits != 32) return HDD_UNSUPPORTED_OUT_NBITS;
  if (nsamps <= (hdd_size)p->max_delay) return HDD_TOO_FEW_NSAMPS;
  if (nsamps > (hdd_size)(65535u * 32u)) return HDD_UNKNOWN_ERROR;  // transpose grid limit
  const int nout = (int)(nsamps - p->max_delay);
  if (in_stride < (hdd_size)p->nchans) return HDD_INVALID_STRIDE;
  if (out_stride % 4 != 0 || out_stride < (hdd_size)nout * 4) return HDD_INVALID_STRIDE;
  if (first_dm_idx + dm_count > p->dms.size() || dm_count == 0) return HDD_UNKNOWN_ERROR;
  if (cudaSetDevice(p->device) != cudaSuccess) return HDD_INVALID_DEVICE_INDEX;
  if (cudaPeekAtLastError() != cudaSuccess) return HDD_PRIOR_GPU_ERROR;
  const bool device = (flags & HDD_DEVICE_POINTERS) != 0;

  hg::DeviceTables tb;
  hdd_error e = hg::plan_device_tables(p, (int)first_dm_idx, (int)dm_count, &tb);
  if (e != HDD_NO_ERROR) return e;
  const uint8_t *din = in;
  const size_t in_bytes = (size_t)(nsamps - 1) * in_stride + p->nchans;
  if (!device) {
    if ((e = grow((void **)&p->d_in, &p->in_cap, in_bytes)) != HDD_NO_ERROR) return e;
    if (cudaMemcpyAsync(p->d_in, in, in_bytes, cudaMemcpyHostToDevice, p->stream) != cudaSuccess)
      return HDD_MEM_COPY_FAILED;
    din = p->d_in;
  }
  const long R = ((long)nsamps + 3) / 4 * 4;
  if ((e = grow((void **)&p->d_plain, &p->plain_cap, (size_t)p->nchans * R)) != HDD_NO_ERROR)
    return e;
  if ((e = grow((void **)&p->d_packed, &p->packed_cap, (size_t)p->nchans * R * 4)) != HDD_NO_ERROR)
    return e;
  float *dout = reinterpret_cast<float *>(out);
  if (!device) {
    if ((e = grow((void **)&p->d_out, &p->out_cap, (size_t)dm_count * out_stride)) != HDD_NO_ERROR)
      return e;
    dout = reinterpret_cast<float *>(p->d_out);
  }
  if (hg::transpose_tf(din, in_stride, (int)nsamps, p->nchans, p->d_plain, R, p->stream) !=
      cudaSuccess)
    return HDD_INTERNAL_GPU_ERROR;
  if (hg::pack_ring(p->d_plain, p->d_packed, 1, p->nchans, R, 0, R, p->stream) != cudaSuccess)
    return HDD_INTERNAL_GPU_ERROR;
  if (!p->d_err) {
    if (cudaMalloc((void **)&p->d_err, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return HDD_MEM_ALLOC_FAILED;
    }
    if (cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) return HDD_INTERNAL_GPU_ERROR;
  }
  const hg::DedispArgs a = hg::single_beam_args(tb, p->d_packed, R, 0, (int)first_dm_idx, (int)dm_count,
                                                nout, dout, (long)(out_stride / 4), p->d_err);
  bool done = false;
  if (a.nact > 0 && p->pair_rows) {  // pair rows, 8 pairs a stage
    hg::PairDeviceTables pt;
    if ((e = hg::plan_pair_tables(p, (int)first_dm_idx, (int)dm_count, 8, hg::dedisp_time_tiles(nout),
                                  p->pair_rows, &pt)) != HDD_NO_ERROR)
      return e;
    hg::DedispArgs pa = hg::single_beam_args(hg::DeviceTables{nullptr, nullptr, hg::kPairDPT, 0, pt.nact, 8},
                                             p->d_packed, R, 0, (int)first_dm_idx, (int)dm_count, nout, dout,
                                             (long)(out_stride / 4), p->d_err);
    hg::use_pair_tables(&pa, pt);
    const cudaError_t ce = hg::dedisperse(pa, p->stream);
    if (ce == cudaSuccess)
      done = true;
    else if (ce == cudaErrorInvalidValue)  // stages beyond shared memory: the channel-by-channel kernel
      cudaGetLastError();
    else
      return HDD_INTERNAL_GPU_ERROR;
  }
  if (done) {
  } else if (a.nact == 0) {
    for (hdd_size d = 0; d < dm_count; ++d)
      if (cudaMemsetAsync(reinterpret_cast<uint8_t *>(dout) + d * out_stride, 0, (size_t)nout * 4,
                          p->stream) != cudaSuccess)
        return HDD_INTERNAL_GPU_ERROR;
  } else if (hg::dedisperse(a, p->stream) != cudaSuccess) {
    return HDD_INTERNAL_GPU_ERROR;
  }
  if (!device) {
    if (cudaMemcpy2DAsync(out, out_stride, dout, out_stride, (size_t)nout * 4, dm_count,
                          cudaMemcpyDeviceToHost, p->stream) != cudaSuccess)
      return HDD_MEM_COPY_FAILED;
  }
  if (!(flags & HDD_ASYNC)) {
    if (cudaStreamSynchronize(p->stream) != cudaSuccess) return HDD_INTERNAL_GPU_ERROR;
    int err = 0;
    if (cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return HDD_INTERNAL_GPU_ERROR;
    if (err) {
      cudaMemset(p->d_err, 0, sizeof(int));
      return HDD_INTERNAL_GPU_ERROR;  // a staging wait timed out
    }
  }
  return HDD_NO_ERROR;
}

hdd_error hdd_execute_adv(hdd_plan p, hdd_size nsamps, const hdd_byte *in, hdd_size in_nbits,
                          hdd_size in_stride, hdd_byte *out, hdd_size out_nbits,
                          hdd_size out_stride, unsigned flags) {
  if (!p) return HDD_INVALID_PLAN;
  return hdd_execute_guru(p, nsamps, in, in_nbits, in_stride, out, out_nbits, out_stride, 0,
                          p->dms.size(), flags);
}

hdd_error hdd_execute(hdd_plan p, hdd_size nsamps, const hdd_byte *in, hdd_size in_nbits,
                      hdd_byte *out, hdd_size out_nbits, unsigned flags) {
  if (!p) return HDD_INVALID_PLAN;
  if (nsamps <= (hdd_size)p->max_delay) return HDD_TOO_FEW_NSAMPS;
  const hdd_size in_stride = (hdd_size)p->nchans * in_nbits / 8;
  const hdd_size out_stride = (nsamps - p->max_delay) * out_nbits / 8;
  return hdd_execute_adv(p, nsamps, in, in_nbits, in_stride, out, out_nbits, out_stride, flags);
}

const char *hdd_get_error_string(hdd_error e) {
  switch (e) {
    case HDD_NO_ERROR: return "no error";
    case HDD_MEM_ALLOC_FAILED: return "mem alloc failed";
    case HDD_MEM_COPY_FAILED: return "mem copy failed";
    case HDD_NCHANS_EXCEEDS_LIMIT: return "nchans exceeds limit";
    case HDD_INVALID_PLAN: return "invalid plan";
    case HDD_INVALID_POINTER: return "invalid pointer";
    case HDD_INVALID_STRIDE: return "invalid stride";
    case HDD_NO_DM_LIST_SET: return "no dm list set";
    case HDD_TOO_FEW_NSAMPS: return "too few nsamps";
    case HDD_INVALID_FLAG_COMBINATION: return "invalid flag combination";
    case HDD_UNSUPPORTED_IN_NBITS: return "unsupported in nbits";
    case HDD_UNSUPPORTED_OUT_NBITS: return "unsupported out nbits";
    case HDD_INVALID_DEVICE_INDEX: return "invalid device index";
    case HDD_DEVICE_ALREADY_SET: return "device already set";
    case HDD_PRIOR_GPU_ERROR: return "prior gpu error";
    case HDD_INTERNAL_GPU_ERROR: return "internal gpu error";
    case HDD_UNKNOWN_ERROR: return "unknown error";
    case HDD_STATIC_SCRATCH_EXCEEDED: return "request exceeds the static scratch of hdd_execute_noalloc";
  }
  return "unknown code";
}

}  // extern "C"
