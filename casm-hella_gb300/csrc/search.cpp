// search.cpp -- the hella_ stage API (include/hella_search.h).
//
// Host orchestration of one search pipeline: what initialize(), the gulp
// loop and the stage functions of casm-hella do
// (src/apps/casm_hella_refactored.cu:54-309 and :659-835), over device
// state that stays resident between gulps.  The overlap carry is a ring of
// NTIME samples per beam: the reference shifts its buffer left by one gulp
// after every gulp (:775-797); here the window start `win0` advances
// instead and the flagger writes each new gulp over the oldest samples.
#include "hella_search.h"
#include "hella_dedisp.h"
#include "hg_internal.h"
#include "hg_plan.h"
#include "hg_search.h"
#include "hg_tune.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

namespace hg {

// smooth.cpp:42-58: 3 x (2sm+1) taps, v from a double expression stored as
// float, products and normalising sum in float.  Returns the middle row.
std::vector<float> middle_taps(int sm) {
  const float wt[3] = {0.3f, 1.f, 0.3f};
  const int n = 2 * sm + 1;
  std::vector<float> k(3 * n);
  float filtSum = 0.f;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < n; ++j) {
      const double u = (j - sm) / (sm / 2.355);
      const float v = (float)(1. - 0.5 * u * u + 0.25 * u * u * 0.25 * u * u -
                              0.083 * u * u * 0.083 * u * u * 0.083 * u * u);
      const float kv = wt[i] * v * v;
      k[i * n + j] = kv;
      filtSum += kv;
    }
  std::vector<float> mid(n);
  for (int j = 0; j < n; ++j) mid[j] = k[n + j] / filtSum;
  return mid;
}

void smoothing_taps(const hella_params &p, int nbox, std::vector<float> *taps, std::vector<int> *off,
                    std::vector<int> *n) {
  taps->clear();
  off->clear();
  n->clear();
  for (int b = 0; b < nbox; ++b) {
    std::vector<float> m = middle_taps(p.width_min << b);
    off->push_back((int)taps->size());
    const int np = ((int)m.size() + 15) / 16 * 16;  // zero padded to a multiple of 16
    n->push_back(np);
    m.resize(np, 0.f);
    taps->insert(taps->end(), m.begin(), m.end());
  }
}

hella_status validate_params(const hella_params *p) {
  if (!p) return HELLA_ERR_INVALID_ARG;
  if (p->nchan < 32 || p->nchan % 32 != 0 || p->nchan > 8192) return HELLA_ERR_INVALID_ARG;
  if (p->nbeam < 1 || p->nbeam > 65535) return HELLA_ERR_INVALID_ARG;
  if (p->gulp < 256 || p->gulp % 32 != 0) return HELLA_ERR_INVALID_ARG;
  if (!(p->tsamp > 0) || !(p->plan_dt > 0) || !(p->f0_mhz > 0) || !(p->df_mhz != 0))
    return HELLA_ERR_INVALID_ARG;
  if (p->f0_mhz - p->nchan * std::abs(p->df_mhz) <= 0) return HELLA_ERR_INVALID_ARG;
  if (!(p->dm_max >= p->dm_min) || p->dm_min < 0 || !(p->dm_tol > 1)) return HELLA_ERR_INVALID_ARG;
  if (p->width_min < 1 || p->width_max <= p->width_min || p->width_max > 4096)
    return HELLA_ERR_INVALID_ARG;
  if (p->max_giants < 1) return HELLA_ERR_INVALID_ARG;
  if (p->smooth_anchor != 0 && p->smooth_anchor != 1) return HELLA_ERR_INVALID_ARG;
  if (p->nscrunch < 0 || p->nscrunch > HELLA_MAX_SCRUNCH) return HELLA_ERR_INVALID_ARG;
  if (p->input_format != HELLA_INPUT_U8_TF && p->input_format != HELLA_INPUT_F16_FT) return HELLA_ERR_INVALID_ARG;
  if (p->bp_median < 1 || p->bp_median % 2 == 0 || p->bp_median > hg::kMaxBpMedian || p->bp_median >= p->nchan)
    return HELLA_ERR_INVALID_ARG;
  if (p->always_find_peaks != 0 && p->always_find_peaks != 1) return HELLA_ERR_INVALID_ARG;
  for (int i = 0; i < p->nscrunch; ++i) {
    const hella_scrunch &sc = p->scrunch[i];
    if (sc.tscrunch < 1 || sc.tscrunch > kMaxScrunch || sc.fscrunch < 1 || sc.fscrunch > kMaxScrunch ||
        !(sc.thresh > 0.f) || !(sc.thresh < 3.0e38f))
      return HELLA_ERR_INVALID_ARG;
  }
  return HELLA_OK;
}

void flag_scrunch_params(const hella_params &p, FlagState *f) {
  f->nscrunch = p.nscrunch;
  for (int i = 0; i < p.nscrunch; ++i) {
    f->sc_t[i] = p.scrunch[i].tscrunch;
    f->sc_f[i] = p.scrunch[i].fscrunch;
    f->sc_thresh[i] = p.scrunch[i].thresh;
  }
  f->flag_lo = p.flag1;
  f->flag_hi = p.flag2;
  f->f16_input = p.input_format == HELLA_INPUT_F16_FT;
  f->bp_median = p.bp_median;
}

size_t gulp_bytes(const hella_params &p) {
  return (size_t)p.nbeam * p.gulp * p.nchan * (p.input_format == HELLA_INPUT_F16_FT ? 2 : 1);
}

}  // namespace hg

struct hella_ctx {
  hella_params p{};
  cudaStream_t stream = nullptr;
  hdd_plan plan = nullptr;
  int ntime = 0, ndms = 0, max_delay = 0, ntime_dd = 0, ntime_out = 0, nbox = 0, min_gulp = 0;
  int gulp_index = 0;
  long R = 0, win0 = 0;
  size_t dev_bytes = 0;
  std::vector<void *> dallocs, hallocs;
  uint8_t *d_gulp = nullptr, *d_plain = nullptr;
  uint32_t *d_packed = nullptr;
  hg::FlagState fs{};
  float *d_dd = nullptr, *d_boxes = nullptr, *d_taps = nullptr;
  int *d_tapoff = nullptr, *d_tapn = nullptr;
  float *d_rowmean = nullptr, *d_rowmax = nullptr, *d_rowvar = nullptr, *d_stats = nullptr,
        *d_gate = nullptr, *d_flagspec = nullptr;
  int *d_counts = nullptr, *d_offsets = nullptr, *d_total = nullptr;
  // one-beam table of the smoothing kernels (updated before each peak pass)
  hg::SmoothBeam *d_sbeam = nullptr, *h_sbeam = nullptr;
  int *d_row_beam = nullptr, *d_active = nullptr;
  int4 *d_cand_i = nullptr;
  float *d_cand_v = nullptr;
  int4 *h_cand_i = nullptr;
  float *h_cand_v = nullptr;
  int *h_total = nullptr;
  std::vector<hella_cand> peaks;
  std::vector<int> tap_n;
  bool loaded = false, flagged = false, smoothed = false;
  int dd_beam = -1;
  int *d_err = nullptr;  // device status word of the staging waits
  hella_tuning tune{0, 4, 8, 0, hg::kDedispGroup, 0};
};

namespace {

const int kOne = 1;

#define CK(x)                                      \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) {                       \
      cudaGetLastError();                          \
      return HELLA_ERR_CUDA;                       \
    }                                              \
  } while (0)

hella_status dalloc(hella_ctx *c, void **ptr, size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  if (cudaMalloc(ptr, bytes) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return HELLA_ERR_ALLOC;
  }
  c->dallocs.push_back(*ptr);
  c->dev_bytes += bytes;
  return HELLA_OK;
}

hella_status halloc(hella_ctx *c, void **ptr, size_t bytes) {
  if (cudaMallocHost(ptr, std::max<size_t>(bytes, 16)) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return HELLA_ERR_ALLOC;
  }
  c->hallocs.push_back(*ptr);
  return HELLA_OK;
}

hg::SmoothArgs smooth_args(hella_ctx *c) {
  hg::SmoothArgs a{};
  a.beams = c->d_sbeam;
  a.nbeam = 1;
  a.row_beam = c->d_row_beam;
  a.nrows = c->ndms - 2;
  a.ntime_dd = c->ntime_dd;
  a.ntime_out = c->ntime_out;
  a.nbox = c->nbox;
  a.wmin = c->p.width_min;
  a.wmax = c->p.width_max;
  a.anchor = c->p.smooth_anchor;
  a.w0 = 0;
  a.nw = c->nbox;
  a.taps = c->d_taps;
  a.tap_off = c->d_tapoff;
  a.tap_n = c->d_tapn;
  a.snr = c->p.snr;
  a.nogate = c->p.always_find_peaks != 0;
  return a;
}

// The context's one-beam smoothing table with candidate cap `cap` and
// reported beam `beam_id`, copied to the device on the context's stream.
hella_status upload_beam(hella_ctx *c, int cap, int beam_id) {
  hg::SmoothBeam &B = *c->h_sbeam;
  B.dd = c->d_dd;
  B.dd_stride = c->ntime_dd;
  B.boxes = c->d_boxes;
  B.rowmean = c->d_rowmean;
  B.rowmax = c->d_rowmax;
  B.rowvar = c->d_rowvar;
  B.stats = c->d_stats;
  B.gate = c->d_gate;
  B.counts = c->d_counts;
  B.offsets = c->d_offsets;
  B.cand_i = c->d_cand_i;
  B.cand_v = c->d_cand_v;
  B.total = c->d_total;
  B.active = c->d_active;
  B.h = c->ndms - 2;
  B.row0 = 0;
  B.cap = cap;
  B.beam_id = beam_id;
  if (cudaMemcpyAsync(c->d_sbeam, c->h_sbeam, sizeof(hg::SmoothBeam), cudaMemcpyHostToDevice,
                      c->stream) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  return HELLA_OK;
}


// Dedisperses `beam`'s window into the plane with tile shape t.
hella_status dedisperse_beam(hella_ctx *c, int beam, const hella_tuning &t) {
  if (!hg::tuning_ok(t)) return HELLA_ERR_INVALID_ARG;
  if (t.add_mode == 4) {  // sub-band sums: tables of their own, 16-trial tiles
    hg::SubDeviceTables sb;
    if (hg::plan_sub_tables(c->plan, 0, c->ndms, &sb) != HDD_NO_ERROR) return HELLA_ERR_DEDISP;
    if (sb.nact == 0) {
      CK(cudaMemsetAsync(c->d_dd, 0, (size_t)c->ndms * c->ntime_dd * 4, c->stream));
      return HELLA_OK;
    }
    const hg::DeviceTables tb{sb.meta, nullptr, hg::kSubDPT, sb.max_spread, sb.nact, hg::kSubG};
    hg::DedispArgs a = hg::single_beam_args(tb, c->d_packed + (size_t)beam * c->p.nchan * c->R, c->R,
                                            c->win0, 0, c->ndms, c->ntime_dd, c->d_dd, c->ntime_dd,
                                            c->d_err);
    hg::use_sub_tables(&a, sb);
    a.group = t.group;
    a.nbuf = t.stages;
    const cudaError_t e = hg::dedisperse(a, c->stream);
    if (e == cudaErrorInvalidValue) {  // the DM list's tiles do not fit this kernel's staging
      cudaGetLastError();
      return HELLA_ERR_INVALID_ARG;
    }
    CK(e);
    return HELLA_OK;
  }
  if (t.add_mode >= 5) {  // rows of channel pairs (5) or quads (6): tables and a row buffer of their own
    const int g = t.add_mode == 6 ? 4 : 2, cc = t.chan_chunk / 2, ntt = hg::dedisp_time_tiles(c->ntime_dd);
    if (c->p.hbm_budget) {  // the rows are not in the creation-time estimate
      size_t bytes = 0;
      if (hg::plan_pair_bytes(c->plan, 0, c->ndms, cc, ntt, g, &bytes) != HDD_NO_ERROR) return HELLA_ERR_DEDISP;
      if (c->dev_bytes + bytes > c->p.hbm_budget) return HELLA_ERR_BUDGET;
    }
    hg::PairDeviceTables pt;
    const hdd_error he = hg::plan_pair_tables(c->plan, 0, c->ndms, cc, ntt, g, &pt);
    if (he == HDD_MEM_ALLOC_FAILED) return HELLA_ERR_ALLOC;
    if (he != HDD_NO_ERROR) return HELLA_ERR_DEDISP;
    if (pt.nact == 0) {
      CK(cudaMemsetAsync(c->d_dd, 0, (size_t)c->ndms * c->ntime_dd * 4, c->stream));
      return HELLA_OK;
    }
    const hg::DeviceTables tb{nullptr, nullptr, hg::kPairDPT, 0, pt.nact, cc};
    hg::DedispArgs a = hg::single_beam_args(tb, c->d_packed + (size_t)beam * c->p.nchan * c->R, c->R,
                                            c->win0, 0, c->ndms, c->ntime_dd, c->d_dd, c->ntime_dd,
                                            c->d_err);
    hg::use_pair_tables(&a, pt);
    a.group = t.group;
    a.nbuf = t.stages;
    const cudaError_t e = hg::dedisperse(a, c->stream);
    if (e == cudaErrorInvalidValue) {  // the DM list's stages do not fit this kernel's staging
      cudaGetLastError();
      return HELLA_ERR_INVALID_ARG;
    }
    CK(e);
    return HELLA_OK;
  }
  hg::DeviceTables tb;
  if (hg::plan_device_tables(c->plan, 0, c->ndms, &tb, t.dm_per_block, t.chan_chunk) != HDD_NO_ERROR)
    return HELLA_ERR_DEDISP;
  if (t.add_mode && tb.dpt < 8) return HELLA_ERR_INVALID_ARG;
  hg::DedispArgs a = hg::single_beam_args(tb, c->d_packed + (size_t)beam * c->p.nchan * c->R, c->R,
                                          c->win0, 0, c->ndms, c->ntime_dd, c->d_dd, c->ntime_dd,
                                          c->d_err);
  a.group = t.group;
  a.nbuf = t.stages;
  a.mode = t.add_mode;
  if (tb.nact == 0)
    CK(cudaMemsetAsync(c->d_dd, 0, (size_t)c->ndms * c->ntime_dd * 4, c->stream));
  else
    CK(hg::dedisperse(a, c->stream));
  return HELLA_OK;
}

// Best of `reps` timed dedispersions of beam 0 with shape t, in ms.
hella_status time_shape(hella_ctx *c, const hella_tuning &t, int reps, float *ms) {
  hella_status s = hg::time_runs(c->stream, reps, [&] { return dedisperse_beam(c, 0, t); }, ms);
  if (s != HELLA_OK) return s;
  int err = 0;
  CK(cudaMemcpy(&err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(c->d_err, 0, sizeof(int));
    return HELLA_ERR_TIMEOUT;
  }
  return HELLA_OK;
}

hella_status autotune(hella_ctx *c, int reps, hella_tuning *out, float *out_ms) {
  hella_tuning best;
  float best_ms = 0.f;
  const hella_status s = hg::tune_shapes(
      c->tune, [&](const hella_tuning &t, float *ms) { return time_shape(c, t, reps, ms); }, &best,
      &best_ms);
  if (s != HELLA_OK) return s;
  c->tune = best;
  if (best.add_mode < 5) hg::plan_pair_release(c->plan);  // the rows are only kept for add modes 5 and 6
  if (out) *out = best;
  if (out_ms) *out_ms = best_ms;
  return HELLA_OK;
}

}  // namespace

extern "C" {

void hella_params_default(hella_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->nchan = 3072;
  p->nbeam = 1;
  p->gulp = 32768;
  p->tsamp = 1.048576e-3;
  p->plan_dt = 1.0e-3;
  p->f0_mhz = 468.75;
  p->df_mhz = -0.03075;
  p->dm_min = 0.f;
  p->dm_max = 100.f;
  p->dm_tol = 1.3f;
  p->ti_us = 40.f;
  p->width_min = 1;
  p->width_max = 128;
  p->snr = 10.f;
  p->spec_min = -0.05f;
  p->spec_max = 0.15f;
  p->flag1 = -1;
  p->flag2 = -1;
  p->max_giants = HELLA_MAX_GIANTS;
  p->smooth_anchor = 1;
  p->bp_median = 1;
}

void hella_destroy(hella_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->p.device);
  cudaStreamSynchronize(c->stream);
  for (void *ptr : c->dallocs) cudaFree(ptr);
  for (void *ptr : c->hallocs) cudaFreeHost(ptr);
  hdd_destroy_plan(c->plan);
  delete c;
}

hella_status hella_create(hella_ctx **out, const hella_params *p) {
  if (!out) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  hella_status st = hg::validate_params(p);
  if (st != HELLA_OK) return st;
  if (cudaSetDevice(p->device) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  hella_ctx *c = new (std::nothrow) hella_ctx;
  if (!c) return HELLA_ERR_ALLOC;
  c->p = *p;
  auto fail = [&](hella_status s) {
    hella_destroy(c);
    return s;
  };
  if (hdd_create_plan(&c->plan, p->nchan, (float)p->plan_dt, (float)p->f0_mhz, (float)p->df_mhz) !=
      HDD_NO_ERROR)
    return fail(HELLA_ERR_DEDISP);
  if (hdd_generate_dm_list(c->plan, p->dm_min, p->dm_max, p->ti_us, p->dm_tol) != HDD_NO_ERROR)
    return fail(HELLA_ERR_DEDISP);
  c->ndms = (int)hdd_get_dm_count(c->plan);
  if (c->ndms < 3) return fail(HELLA_ERR_INVALID_ARG);
  c->max_delay = (int)hdd_get_max_delay(c->plan);
  c->ntime = 32 * ((p->gulp + c->max_delay + p->width_max) / 32 + 1);  // :217-219
  c->R = c->ntime;
  c->ntime_dd = p->gulp + p->width_max;
  c->ntime_out = p->gulp;
  for (int sm = p->width_min; sm < p->width_max; sm *= 2) c->nbox++;
  c->min_gulp = c->ntime / p->gulp;  // :632

  const size_t nb = p->nbeam, nch = p->nchan, R = c->R, h = c->ndms - 2;
  const size_t need = nb * p->gulp * nch + nb * nch * R * 5 + nb * nch * (256 * 6 + 16) +
                      (p->nscrunch > 0 || p->input_format ? nb * nch * (p->gulp * 6 + 8) : 0) +
                      (p->input_format ? nb * p->gulp * nch : 0) +
                      nb * p->gulp * 6 + (size_t)c->ndms * c->ntime_dd * 4 +
                      (size_t)c->nbox * h * c->ntime_out * 4 + (size_t)c->nbox * h * 20 +
                      (size_t)p->max_giants * 20;
  if (p->hbm_budget && need > p->hbm_budget) return fail(HELLA_ERR_BUDGET);

  hella_status s;
#define DA(ptr, bytes)                                                  \
  if ((s = dalloc(c, (void **)&(ptr), (bytes))) != HELLA_OK) return fail(s);
  DA(c->d_gulp, hg::gulp_bytes(*p));
  DA(c->d_plain, nb * nch * R);
  DA(c->d_packed, nb * nch * R * 4);
  hg::FlagState &f = c->fs;
  f.nbeam = p->nbeam;
  f.nchan = p->nchan;
  f.gulp = p->gulp;
  f.spec_min = p->spec_min;
  f.spec_max = p->spec_max;
  DA(f.bp1, nb * nch * 4);
  DA(f.bp2, nb * nch * 4);
  DA(f.bp3, nb * nch * 4);
  DA(f.part, nb * nch * 256 * 4);
  DA(f.rowval, nb * nch * 4);
  DA(f.scal, nb * 8 * 4);
  DA(f.hsc, nb * 8 * 2);
  DA(f.lut, nb * nch * 256 * 2);
  DA(f.flag2, nb * nch);
  DA(f.ts, nb * p->gulp * 4);
  DA(f.hts, nb * p->gulp * 2);
  hg::flag_scrunch_params(*p, &f);
  if (p->nscrunch > 0 || f.f16_input) {
    DA(f.P, nb * nch * p->gulp * 2);
    DA(f.M, nb * nch * p->gulp * 2);
    DA(f.S, nb * nch * p->gulp * 2);
    DA(f.bpx, nb * nch * 4);
    DA(f.fsb, nb * nch * 4);
  }
  DA(c->d_dd, (size_t)c->ndms * c->ntime_dd * 4);
  DA(c->d_boxes, (size_t)c->nbox * h * c->ntime_out * 4);
  DA(c->d_rowmean, c->nbox * h * 4);
  DA(c->d_rowmax, c->nbox * h * 4);
  DA(c->d_rowvar, c->nbox * h * 4);
  DA(c->d_stats, c->nbox * 16);
  DA(c->d_gate, 16);
  DA(c->d_flagspec, nch * 4);
  f.flagspec = c->d_flagspec;
  DA(c->d_counts, c->nbox * h * 4);
  DA(c->d_offsets, c->nbox * h * 4);
  DA(c->d_total, 16);
  DA(c->d_cand_i, (size_t)p->max_giants * 16);
  DA(c->d_cand_v, (size_t)p->max_giants * 4);
  DA(c->d_err, 16);
  DA(c->d_sbeam, sizeof(hg::SmoothBeam));
  DA(c->d_row_beam, (size_t)c->ndms * 4);
  DA(c->d_active, 16);
#undef DA
  if ((s = halloc(c, (void **)&c->h_cand_i, (size_t)p->max_giants * 16)) != HELLA_OK) return fail(s);
  if ((s = halloc(c, (void **)&c->h_cand_v, (size_t)p->max_giants * 4)) != HELLA_OK) return fail(s);
  if ((s = halloc(c, (void **)&c->h_total, 16)) != HELLA_OK) return fail(s);
  if ((s = halloc(c, (void **)&c->h_sbeam, sizeof(hg::SmoothBeam))) != HELLA_OK) return fail(s);

  // smoothing taps: middle rows, zero padded to a multiple of 16
  std::vector<float> taps;
  std::vector<int> off, n;
  hg::smoothing_taps(*p, c->nbox, &taps, &off, &n);
  c->tap_n = n;
  if ((s = dalloc(c, (void **)&c->d_taps, taps.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(c, (void **)&c->d_tapoff, off.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(c, (void **)&c->d_tapn, n.size() * 4)) != HELLA_OK) return fail(s);
  if (cudaMemcpy(c->d_taps, taps.data(), taps.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_tapoff, off.data(), off.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_tapn, n.data(), n.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(c->d_plain, 0, nb * nch * R) != cudaSuccess ||
      cudaMemset(c->d_packed, 0, nb * nch * R * 4) != cudaSuccess ||
      cudaMemset(c->d_flagspec, 0, nch * 4) != cudaSuccess ||
      cudaMemset(c->d_err, 0, 16) != cudaSuccess ||
      cudaMemset(c->d_row_beam, 0, (size_t)c->ndms * 4) != cudaSuccess ||
      cudaMemcpy(c->d_active, &kOne, 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_CUDA);
  }
  if ((s = upload_beam(c, p->max_giants, p->beam0)) != HELLA_OK) return fail(s);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(HELLA_ERR_CUDA);
  if (p->autotune && (s = autotune(c, 2, nullptr, nullptr)) != HELLA_OK) return fail(s);
  *out = c;
  return HELLA_OK;
}

hella_status hella_set_stream(hella_ctx *c, void *stream) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  c->stream = (cudaStream_t)stream;
  hdd_set_stream(c->plan, stream);
  return HELLA_OK;
}

hella_status hella_get_info(const hella_ctx *c, hella_info *i) {
  if (!c || !i) return HELLA_ERR_INVALID_ARG;
  i->ntime = c->ntime;
  i->ndms = c->ndms;
  i->max_delay = c->max_delay;
  i->ntime_dd = c->ntime_dd;
  i->ntime_out = c->ntime_out;
  i->nboxcar = c->nbox;
  i->min_gulp = c->min_gulp;
  i->gulp_index = c->gulp_index;
  i->device_bytes = c->dev_bytes;
  return HELLA_OK;
}

const float *hella_get_dm_list(const hella_ctx *c) { return c ? hdd_get_dm_list(c->plan) : nullptr; }

hella_status hella_set_killmask(hella_ctx *c, const int *killmask) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  return hdd_set_killmask(c->plan, killmask) == HDD_NO_ERROR ? HELLA_OK : HELLA_ERR_DEDISP;
}

hella_status hella_load_gulp(hella_ctx *c, const uint8_t *gulp, int on_device) {
  if (!c || !gulp) return HELLA_ERR_INVALID_ARG;
  const size_t n = hg::gulp_bytes(c->p);
  CK(cudaMemcpyAsync(c->d_gulp, gulp, n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     c->stream));
  c->loaded = true;
  return HELLA_OK;
}

hella_status hella_fast_flagger(hella_ctx *c) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  if (!c->loaded) return HELLA_ERR_STATE;
  const long wpos = (c->win0 + c->R - c->p.gulp) % c->R;
  CK(hg::flag_gulp(c->fs, c->d_gulp, c->d_plain, c->R, wpos, c->stream));
  CK(hg::pack_ring(c->d_plain, c->d_packed, c->p.nbeam, c->p.nchan, c->R, wpos - 3L * hg::kPackS,
                   c->p.gulp + 3L * hg::kPackS, c->stream));
  c->flagged = true;
  return HELLA_OK;
}

hella_status hella_dedisperse(hella_ctx *c, int beam) {
  if (!c || beam < 0 || beam >= c->p.nbeam) return HELLA_ERR_INVALID_ARG;
  if (!c->flagged) return HELLA_ERR_STATE;
  hella_status s = dedisperse_beam(c, beam, c->tune);
  if (s != HELLA_OK) return s;
  c->dd_beam = beam;
  c->smoothed = false;
  return HELLA_OK;
}

hella_status hella_smooth(hella_ctx *c, int scale) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  if (c->dd_beam < 0) return HELLA_ERR_STATE;
  const hg::SmoothArgs a = smooth_args(c);
  CK(hg::smooth_planes(a, c->stream));
  if (scale) {
    CK(hg::smooth_stats(a, c->stream, 1));
  } else {
    CK(hg::smooth_stats(a, c->stream, 0));
  }
  c->smoothed = true;
  return HELLA_OK;
}

hella_status hella_find_peaks(hella_ctx *c, int beam) {
  if (!c || beam < 0 || beam >= c->p.nbeam) return HELLA_ERR_INVALID_ARG;
  if (!c->smoothed) return HELLA_ERR_STATE;
  const int cap = c->p.max_giants - (int)c->peaks.size();
  if (cap <= 0) return HELLA_OK;
  hella_status st = upload_beam(c, cap, beam + c->p.beam0);
  if (st != HELLA_OK) return st;
  CK(cudaMemsetAsync(c->d_total, 0, 4, c->stream));
  CK(hg::find_peaks(smooth_args(c), c->stream));
  CK(cudaMemcpyAsync(c->h_total, c->d_total, 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_total + 1, c->d_err, 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->h_total[1]) {  // a dedispersion staging wait timed out
    cudaMemsetAsync(c->d_err, 0, 4, c->stream);
    return HELLA_ERR_TIMEOUT;
  }
  const int n = std::min(*c->h_total, cap);
  if (n > 0) {
    CK(cudaMemcpyAsync(c->h_cand_i, c->d_cand_i, (size_t)n * 16, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(c->h_cand_v, c->d_cand_v, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < n; ++i) {
      hella_cand h;
      h.beam = c->h_cand_i[i].x;
      h.dm_idx = c->h_cand_i[i].y;
      h.width = c->h_cand_i[i].z;
      h.samp = c->h_cand_i[i].w;
      h.snr = c->h_cand_v[i];
      c->peaks.push_back(h);
    }
  }
  return HELLA_OK;
}

hella_status hella_clear_peaks(hella_ctx *c) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  c->peaks.clear();
  return HELLA_OK;
}

hella_status hella_rewind(hella_ctx *c) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  c->win0 = (c->win0 + c->p.gulp) % c->R;
  c->gulp_index++;
  c->loaded = c->flagged = c->smoothed = false;
  c->dd_beam = -1;
  return HELLA_OK;
}

hella_status hella_get_peaks(hella_ctx *c, hella_cand *out, int max, int *n) {
  if (!c || !n) return HELLA_ERR_INVALID_ARG;
  const int k = std::min((int)c->peaks.size(), std::max(0, max));
  if (k && !out) return HELLA_ERR_INVALID_ARG;
  for (int i = 0; i < k; ++i) out[i] = c->peaks[i];
  *n = k;
  return HELLA_OK;
}

hella_status hella_process_gulp(hella_ctx *c, const uint8_t *gulp, int on_device, hella_cand *out,
                                int max, int *n, int *searched) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  hella_status s;
  if ((s = hella_clear_peaks(c)) != HELLA_OK) return s;
  if ((s = hella_load_gulp(c, gulp, on_device)) != HELLA_OK) return s;
  if ((s = hella_fast_flagger(c)) != HELLA_OK) return s;
  const int do_search = c->gulp_index >= c->min_gulp;  // :705
  if (do_search)
    for (int b = 0; b < c->p.nbeam && (int)c->peaks.size() < c->p.max_giants; ++b) {  // :723
      if ((s = hella_dedisperse(c, b)) != HELLA_OK) return s;
      if ((s = hella_smooth(c, 1)) != HELLA_OK) return s;
      if ((s = hella_find_peaks(c, b)) != HELLA_OK) return s;
    }
  if (searched) *searched = do_search;
  int k = 0;
  if (n) {
    if ((s = hella_get_peaks(c, out, max, &k)) != HELLA_OK) return s;
    *n = k;
  }
  if (!do_search) CK(cudaStreamSynchronize(c->stream));
  return hella_rewind(c);
}

hella_status hella_copy_window(hella_ctx *c, int beam, uint8_t *out) {
  if (!c || !out || beam < 0 || beam >= c->p.nbeam) return HELLA_ERR_INVALID_ARG;
  const size_t nch = c->p.nchan, R = c->R;
  std::vector<uint8_t> tmp(nch * R);
  CK(cudaMemcpyAsync(tmp.data(), c->d_plain + (size_t)beam * nch * R, nch * R, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (size_t t = 0; t < (size_t)c->ntime; ++t) {
    const size_t q = (c->win0 + t) % R;
    for (size_t ch = 0; ch < nch; ++ch) out[t * nch + ch] = tmp[ch * R + q];
  }
  return HELLA_OK;
}

hella_status hella_copy_dedisp(hella_ctx *c, float *out) {
  if (!c || !out) return HELLA_ERR_INVALID_ARG;
  CK(cudaMemcpyAsync(out, c->d_dd, (size_t)c->ndms * c->ntime_dd * 4, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return HELLA_OK;
}

hella_status hella_copy_boxes(hella_ctx *c, float *out) {
  if (!c || !out) return HELLA_ERR_INVALID_ARG;
  const size_t plane = (size_t)(c->ndms - 2) * c->ntime_out;
  std::vector<float> st(c->nbox * 4);
  CK(cudaMemcpyAsync(out, c->d_boxes, plane * c->nbox * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(st.data(), c->d_stats, st.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int b = 0; b < c->nbox; ++b) {
    if (!(st[b * 4 + 1] > 0.f)) continue;
    const float nm = st[b * 4 + 2], rs = st[b * 4 + 3];
    float *x = out + b * plane;
    for (size_t i = 0; i < plane; ++i) {
      const float v = x[i] + nm;
      x[i] = v * rs;
    }
  }
  return HELLA_OK;
}

hella_status hella_get_smooth_stats(hella_ctx *c, float *mean, float *std, float *sigma0) {
  if (!c) return HELLA_ERR_INVALID_ARG;
  std::vector<float> st(c->nbox * 4), g(4);
  CK(cudaMemcpyAsync(st.data(), c->d_stats, st.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(g.data(), c->d_gate, 16, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int b = 0; b < c->nbox; ++b) {
    if (mean) mean[b] = st[b * 4 + 0];
    if (std) std[b] = st[b * 4 + 1];
  }
  if (sigma0) *sigma0 = g[1];
  return HELLA_OK;
}

hella_status hella_get_flag_stats(hella_ctx *c, int beam, float *bp1, float *bp2, float *bp3,
                                  float *scalars, float *ts) {
  if (!c || beam < 0 || beam >= c->p.nbeam) return HELLA_ERR_INVALID_ARG;
  const size_t nch = c->p.nchan, off = (size_t)beam * nch;
  if (bp1) CK(cudaMemcpyAsync(bp1, c->fs.bp1 + off, nch * 4, cudaMemcpyDeviceToHost, c->stream));
  if (bp2) CK(cudaMemcpyAsync(bp2, c->fs.bp2 + off, nch * 4, cudaMemcpyDeviceToHost, c->stream));
  if (bp3) CK(cudaMemcpyAsync(bp3, c->fs.bp3 + off, nch * 4, cudaMemcpyDeviceToHost, c->stream));
  if (ts)
    CK(cudaMemcpyAsync(ts, c->fs.ts + (size_t)beam * c->p.gulp, (size_t)c->p.gulp * 4,
                       cudaMemcpyDeviceToHost, c->stream));
  float sc[8];
  CK(cudaMemcpyAsync(sc, c->fs.scal + beam * 8, 32, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (scalars)
    for (int i = 0; i < 4; ++i) scalars[i] = sc[i];
  return HELLA_OK;
}

hella_status hella_get_flag_spec(hella_ctx *c, float *out) {
  if (!c || !out) return HELLA_ERR_INVALID_ARG;
  CK(cudaMemcpyAsync(out, c->d_flagspec, (size_t)c->p.nchan * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return HELLA_OK;
}

hella_status hella_get_tuning(const hella_ctx *c, hella_tuning *t) {
  if (!c || !t) return HELLA_ERR_INVALID_ARG;
  *t = c->tune;
  return HELLA_OK;
}

hella_status hella_set_tuning(hella_ctx *c, const hella_tuning *t) {
  if (!c || !t || !hg::tuning_ok(*t)) return HELLA_ERR_INVALID_ARG;
  c->tune = *t;
  c->tune.samples_per_thread = 4;
  if (t->add_mode < 5) hg::plan_pair_release(c->plan);
  return HELLA_OK;
}

hella_status hella_time_dedisp(hella_ctx *c, const hella_tuning *t, int reps, float *ms) {
  if (!c || !ms || reps < 1) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->p.device));
  return time_shape(c, t ? *t : c->tune, reps, ms);
}

hella_status hella_autotune(hella_ctx *c, int reps, hella_tuning *best, float *best_ms) {
  if (!c || reps < 1) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->p.device));
  return autotune(c, reps, best, best_ms);
}

const char *hella_status_string(hella_status s) {
  switch (s) {
    case HELLA_OK: return "ok";
    case HELLA_ERR_INVALID_ARG: return "invalid argument";
    case HELLA_ERR_ALLOC: return "allocation failed";
    case HELLA_ERR_CUDA: return "cuda error";
    case HELLA_ERR_STATE: return "stage called out of order";
    case HELLA_ERR_DEDISP: return "dedispersion plan error";
    case HELLA_ERR_BUDGET: return "hbm budget exceeded";
    case HELLA_ERR_TIMEOUT: return "device wait timed out";
    case HELLA_ERR_IO: return "socket error";
  }
  return "unknown status";
}

}  // extern "C"
