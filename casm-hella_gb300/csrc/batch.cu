// batch.cu -- the batched multi-beam search (hella_batch_*, include/hella_search.h).
//
// What casm-hella's gulp loop does beam after beam
// (src/apps/casm_hella_refactored.cu:701-797: fast_flagger for all beams,
// then dedisperse / smooth / find_peaks per beam, then the overlap shift),
// here for every beam at once: each stage is one launch over all beams (one
// per smoothing-width pass), and the whole per-gulp sequence is captured
// once in a CUDA graph and replayed.  Per-gulp values (ring positions, which
// beams are searched, candidate counts) live in device memory, so the graph
// never changes between gulps.
//
// Beams share one ring of R = max over beams of NTIME_b samples.  Beam b's
// single-beam context would keep a ring of NTIME_b samples whose window
// holds the newest NTIME_b samples; the batch reads the same samples at
// window start (win0 + R - NTIME_b) mod R of the shared ring.  A beam's DM
// list is the prefix of the longest one (the list is generated trial after
// trial up to the ceiling), so one set of dedispersion tables serves every
// beam, each beam computing its own number of trials.  Killed channels are
// packed as zeros, which drops them from the exact integer sums.
#include "hella_dedisp.h"
#include "hella_search.h"
#include "hg_internal.h"
#include "hg_plan.h"
#include "hg_search.h"
#include "hg_tune.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

namespace {

// Ring positions and per-beam state of the gulp about to be processed.
__global__ void k_advance(hg::GulpPos *pos, hg::DedispBeam *db, int *active, int *total,
                          const int *ntime_b, const int *min_gulp_b, int nbeam, long R, int gulp) {
  const long win0 = pos->win0;
  const int gi = pos->gulp_index;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) pos->wpos = (win0 + R - gulp) % R;
  if (b < nbeam) {
    db[b].win0 = (win0 + R - ntime_b[b]) % R;
    active[b] = gi >= min_gulp_b[b];  // casm_hella_refactored.cu:705
    total[b] = 0;
  }
}

// The overlap shift (casm_hella_refactored.cu:775-797) as a ring advance.
__global__ void k_rewind(hg::GulpPos *pos, long R, int gulp) {
  pos->win0 = (pos->win0 + gulp) % R;
  pos->gulp_index += 1;
}

// Beam b's candidates into out[sum of the earlier beams' counts ...].
__global__ void k_gather(const hg::SmoothBeam *sb, const int *total, int nbeam, hella_cand *out) {
  __shared__ int off_s[256];
  const int b = blockIdx.x, tid = threadIdx.x;
  int part = 0;
  for (int i = tid; i < b; i += blockDim.x) part += total[i];
  off_s[tid] = part;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (tid < s) off_s[tid] += off_s[tid + s];
    __syncthreads();
  }
  const int off = off_s[0], n = total[b];
  const hg::SmoothBeam &B = sb[b];
  for (int i = tid; i < n; i += blockDim.x) {
    const int4 ci = B.cand_i[i];
    hella_cand c;
    c.beam = ci.x;
    c.dm_idx = ci.y;
    c.width = ci.z;
    c.samp = ci.w;
    c.snr = B.cand_v[i];
    out[off + i] = c;
  }
}

}  // namespace

struct hella_batch {
  hella_params p{};
  int nbeam = 0;
  cudaStream_t stream = nullptr;  // graph capture needs a stream other than the legacy one
  cudaStream_t own_stream = nullptr;
  hdd_plan plan = nullptr;  // the longest DM list; all channels active
  int ndms_all = 0, nbox = 0, ntime_dd = 0, ntime_out = 0, nwp = 1, nrows = 0;
  long R = 0;
  std::vector<int> ndms, max_delay, ntime, min_gulp;
  int gulp_index = 0;
  size_t dev_bytes = 0;
  std::vector<void *> dallocs, hallocs;
  uint8_t *d_gulp = nullptr, *d_plain = nullptr, *d_keep = nullptr;
  uint32_t *d_packed = nullptr;
  hg::FlagState fs{};
  float *d_dd = nullptr, *d_boxes = nullptr, *d_taps = nullptr;
  int *d_tapoff = nullptr, *d_tapn = nullptr;
  float *d_rowmean = nullptr, *d_rowmax = nullptr, *d_rowvar = nullptr, *d_stats = nullptr,
        *d_gate = nullptr;
  int *d_counts = nullptr, *d_offsets = nullptr, *d_total = nullptr, *d_active = nullptr,
      *d_row_beam = nullptr, *d_err = nullptr, *d_ntime = nullptr, *d_min_gulp = nullptr;
  int4 *d_cand_i = nullptr;
  float *d_cand_v = nullptr;
  hella_cand *d_out = nullptr;
  hg::DedispBeam *d_dbeams = nullptr;
  hg::SmoothBeam *d_sbeams = nullptr;
  hg::GulpPos *d_pos = nullptr;
  int *h_total = nullptr;
  std::vector<hg::DedispBeam> dbeams;
  int items_dpt = -1;  // DM tile of the work-item prefix held in d_dbeams
  hella_tuning tune{0, 4, 8, 0, hg::kDedispGroup, 0};
  bool use_graph = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_stale = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
};

namespace {

#define CK(x)                 \
  do {                        \
    if ((x) != cudaSuccess) { \
      cudaGetLastError();     \
      return HELLA_ERR_CUDA;  \
    }                         \
  } while (0)

hella_status dalloc(hella_batch *b, void **ptr, size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  if (cudaMalloc(ptr, bytes) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return HELLA_ERR_ALLOC;
  }
  b->dallocs.push_back(*ptr);
  b->dev_bytes += bytes;
  return HELLA_OK;
}

// Dedispersion launch over all beams with tile shape t (tables uploaded).
hella_status dedisp_args(hella_batch *b, const hella_tuning &t, hg::DedispArgs *out) {
  if (!hg::tuning_ok(t)) return HELLA_ERR_INVALID_ARG;
  hg::DeviceTables tb;
  if (hg::plan_device_tables(b->plan, 0, b->ndms_all, &tb, t.dm_per_block, t.chan_chunk) != HDD_NO_ERROR)
    return HELLA_ERR_DEDISP;
  if (t.add_mode && tb.dpt < 8) return HELLA_ERR_INVALID_ARG;
  hg::DedispArgs a{};
  a.beams = b->d_dbeams;
  a.nbeam = b->nbeam;
  a.ntt = hg::dedisp_time_tiles(b->ntime_dd);
  // work-item prefix of this DM tile (win0 is rewritten on the device each gulp)
  int items = 0;
  for (int i = 0; i < b->nbeam; ++i) {
    b->dbeams[i].item0 = items;
    items += hg::dedisp_items(b->ndms[i], tb.dpt, a.ntt);
  }
  if (b->items_dpt != tb.dpt) {
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaMemcpy(b->d_dbeams, b->dbeams.data(), sizeof(hg::DedispBeam) * b->nbeam, cudaMemcpyHostToDevice));
    b->items_dpt = tb.dpt;
  }
  a.nitems = items;
  a.group = t.group;
  a.R = b->R;
  a.nact = tb.nact;
  a.dm_first = 0;
  a.nout = b->ntime_dd;
  a.out_stride = b->ntime_dd;
  a.dpt = tb.dpt;
  a.cc = tb.cc;
  a.nbuf = t.stages;
  a.mode = t.add_mode;
  a.unit = 1;
  a.max_spread = tb.max_spread;
  a.tile_meta = tb.meta;
  a.tile_off = tb.off;
  a.err = b->d_err;
  *out = a;
  return HELLA_OK;
}

hg::SmoothArgs smooth_args(hella_batch *b, int w0, int nw) {
  hg::SmoothArgs a{};
  a.beams = b->d_sbeams;
  a.nbeam = b->nbeam;
  a.row_beam = b->d_row_beam;
  a.nrows = b->nrows;
  a.ntime_dd = b->ntime_dd;
  a.ntime_out = b->ntime_out;
  a.nbox = b->nbox;
  a.wmin = b->p.width_min;
  a.wmax = b->p.width_max;
  a.anchor = b->p.smooth_anchor;
  a.w0 = w0;
  a.nw = nw;
  a.taps = b->d_taps;
  a.tap_off = b->d_tapoff;
  a.tap_n = b->d_tapn;
  a.snr = b->p.snr;
  return a;
}

// Every launch of one gulp, in order, on b->stream (captured or not).
hella_status enqueue_gulp(hella_batch *b, const hg::DedispArgs &da) {
  const int nb = b->nbeam;
  k_advance<<<(nb + 255) / 256, 256, 0, b->stream>>>(b->d_pos, b->d_dbeams, b->d_active, b->d_total,
                                                     b->d_ntime, b->d_min_gulp, nb, b->R, b->p.gulp);
  CK(hg::flag_gulp_dev(b->fs, b->d_gulp, b->d_plain, b->R, b->d_pos, b->stream));
  CK(hg::pack_gulp_dev(b->d_plain, b->d_packed, nb, b->p.nchan, b->R, b->p.gulp, b->d_pos, b->stream,
                       b->d_keep));
  CK(hg::dedisperse(da, b->stream));
  for (int w0 = 0; w0 < b->nbox; w0 += b->nwp) {
    const hg::SmoothArgs a = smooth_args(b, w0, std::min(b->nwp, b->nbox - w0));
    CK(hg::smooth_planes(a, b->stream));
    CK(hg::smooth_stats(a, b->stream, 1));
    CK(hg::find_peaks(a, b->stream));
  }
  k_gather<<<nb, 256, 0, b->stream>>>(b->d_sbeams, b->d_total, nb, b->d_out);
  CK(cudaMemcpyAsync(b->h_total, b->d_total, sizeof(int) * nb, cudaMemcpyDeviceToHost, b->stream));
  k_rewind<<<1, 1, 0, b->stream>>>(b->d_pos, b->R, b->p.gulp);
  hg::count_launches(3);
  CK(cudaGetLastError());
  return HELLA_OK;
}

// Captures the gulp sequence into the executable graph (first use, or after
// the tile shape or stream changed).
hella_status build_graph(hella_batch *b, const hg::DedispArgs &da) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const hella_status s = enqueue_gulp(b, da);
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (s != HELLA_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return s != HELLA_OK ? s : HELLA_ERR_CUDA;
  }
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = g;
  const cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
  if (ie != cudaSuccess) {
    cudaGetLastError();
    b->exec = nullptr;
    return HELLA_ERR_CUDA;
  }
  b->graph_stale = false;
  return HELLA_OK;
}

hella_status time_shape(hella_batch *b, const hella_tuning &t, int reps, float *ms) {
  hg::DedispArgs da;
  hella_status s = dedisp_args(b, t, &da);
  if (s != HELLA_OK) return s;
  s = hg::time_runs(b->stream, reps, [&]() -> hella_status {
    CK(hg::dedisperse(da, b->stream));
    return HELLA_OK;
  }, ms);
  if (s != HELLA_OK) return s;
  int err = 0;
  CK(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(b->d_err, 0, sizeof(int));
    return HELLA_ERR_TIMEOUT;
  }
  return HELLA_OK;
}

hella_status autotune(hella_batch *b, int reps, hella_tuning *out, float *out_ms) {
  hella_tuning best;
  float best_ms = 0.f;
  const hella_status s = hg::tune_shapes(
      b->tune, [&](const hella_tuning &t, float *ms) { return time_shape(b, t, reps, ms); }, &best,
      &best_ms);
  if (s != HELLA_OK) return s;
  b->tune = best;
  b->graph_stale = true;
  if (out) *out = best;
  if (out_ms) *out_ms = best_ms;
  return HELLA_OK;
}

}  // namespace

extern "C" {

void hella_batch_params_default(hella_batch_params *p) {
  std::memset(p, 0, sizeof(*p));
  hella_params_default(&p->base);
  p->use_graph = 1;
}

void hella_batch_destroy(hella_batch *b) {
  if (!b) return;
  cudaSetDevice(b->p.device);
  cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (void *ptr : b->dallocs) cudaFree(ptr);
  for (void *ptr : b->hallocs) cudaFreeHost(ptr);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  hdd_destroy_plan(b->plan);
  delete b;
}

hella_status hella_batch_create(hella_batch **out, const hella_batch_params *bp) {
  if (!out || !bp) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  const hella_params *p = &bp->base;
  hella_status s = hg::validate_params(p);
  if (s != HELLA_OK) return s;
  if (bp->widths_per_pass < 0) return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(p->device) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  hella_batch *b = new (std::nothrow) hella_batch;
  if (!b) return HELLA_ERR_ALLOC;
  b->p = *p;
  b->nbeam = p->nbeam;
  b->use_graph = bp->use_graph != 0;
  auto fail = [&](hella_status st) {
    hella_batch_destroy(b);
    return st;
  };
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_CUDA);
  }
  b->stream = b->own_stream;
  const int nb = b->nbeam, nch = p->nchan;

  // DM lists: beam b's is the prefix of the longest one up to its ceiling
  std::vector<float> ceil(nb, p->dm_max);
  if (bp->dm_max)
    for (int i = 0; i < nb; ++i) ceil[i] = bp->dm_max[i];
  float top = ceil[0];
  for (float c : ceil) {
    if (!(c >= p->dm_min)) return fail(HELLA_ERR_INVALID_ARG);
    top = std::max(top, c);
  }
  if (hdd_create_plan(&b->plan, nch, (float)p->plan_dt, (float)p->f0_mhz, (float)p->df_mhz) != HDD_NO_ERROR ||
      hdd_generate_dm_list(b->plan, p->dm_min, top, p->ti_us, p->dm_tol) != HDD_NO_ERROR)
    return fail(HELLA_ERR_DEDISP);
  b->ndms_all = (int)hdd_get_dm_count(b->plan);
  const float *all = hdd_get_dm_list(b->plan);
  const int *delays = hdd_get_delay_table(b->plan);
  b->ndms.resize(nb);
  b->max_delay.resize(nb);
  b->ntime.resize(nb);
  b->min_gulp.resize(nb);
  for (int i = 0; i < nb; ++i) {
    const std::vector<float> mine = hg::generate_dm_list(
        (float)p->dm_min, (float)ceil[i], (float)p->ti_us, (float)p->dm_tol, nch, (float)p->plan_dt,
        (float)p->f0_mhz, (float)p->df_mhz);
    if ((int)mine.size() > b->ndms_all || (int)mine.size() < 3) return fail(HELLA_ERR_INVALID_ARG);
    for (size_t k = 0; k < mine.size(); ++k)
      if (mine[k] != all[k]) return fail(HELLA_ERR_DEDISP);  // not a prefix: cannot share tables
    b->ndms[i] = (int)mine.size();
    b->max_delay[i] = delays[(size_t)(b->ndms[i] - 1) * nch + nch - 1];
    b->ntime[i] = 32 * ((p->gulp + b->max_delay[i] + p->width_max) / 32 + 1);  // :217-219
    b->min_gulp[i] = b->ntime[i] / p->gulp;                                      // :632
    b->R = std::max<long>(b->R, b->ntime[i]);
  }
  b->ntime_dd = p->gulp + p->width_max;
  b->ntime_out = p->gulp;
  for (int sm = p->width_min; sm < p->width_max; sm *= 2) b->nbox++;
  std::vector<int> row0(nb);
  for (int i = 0; i < nb; ++i) {
    row0[i] = b->nrows;
    b->nrows += b->ndms[i] - 2;
  }
  size_t dd_floats = 0;
  for (int i = 0; i < nb; ++i) dd_floats += (size_t)b->ndms[i] * b->ntime_dd;

  // HBM: everything but the smoothed planes, then as many widths per pass
  // as the budget allows
  const size_t R = b->R, cap = p->max_giants;
  const size_t fixed = (size_t)nb * p->gulp * nch + (size_t)nb * nch * R * 5 + (size_t)nb * nch +
                       (size_t)nb * nch * (256 * 6 + 16) + (size_t)nb * p->gulp * 6 + dd_floats * 4 +
                       (size_t)b->nrows * b->nbox * 20 + (size_t)nb * (cap * 40 + 256);
  const size_t per_width = (size_t)b->nrows * b->ntime_out * 4;
  size_t budget = p->hbm_budget;
  if (!budget) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return fail(HELLA_ERR_CUDA);
    budget = fr > (1ul << 30) ? fr - (1ul << 30) : 0;  // leave 1 GB to the runtime
  }
  if (fixed + per_width > budget) return fail(HELLA_ERR_BUDGET);
  b->nwp = bp->widths_per_pass ? std::min(bp->widths_per_pass, b->nbox)
                               : (int)std::min<size_t>(b->nbox, (budget - fixed) / per_width);
  if (b->nwp < 1 || fixed + per_width * b->nwp > budget) return fail(HELLA_ERR_BUDGET);

#define DA(ptr, bytes)                                                  \
  if ((s = dalloc(b, (void **)&(ptr), (bytes))) != HELLA_OK) return fail(s);
  DA(b->d_gulp, (size_t)nb * p->gulp * nch);
  DA(b->d_plain, (size_t)nb * nch * R);
  DA(b->d_packed, (size_t)nb * nch * R * 4);
  DA(b->d_keep, (size_t)nb * nch);
  hg::FlagState &f = b->fs;
  f.nbeam = nb;
  f.nchan = nch;
  f.gulp = p->gulp;
  f.spec_min = p->spec_min;
  f.spec_max = p->spec_max;
  DA(f.bp1, (size_t)nb * nch * 4);
  DA(f.bp2, (size_t)nb * nch * 4);
  DA(f.bp3, (size_t)nb * nch * 4);
  DA(f.part, (size_t)nb * nch * 256 * 4);
  DA(f.rowval, (size_t)nb * nch * 4);
  DA(f.scal, (size_t)nb * 8 * 4);
  DA(f.hsc, (size_t)nb * 8 * 2);
  DA(f.lut, (size_t)nb * nch * 256 * 2);
  DA(f.flag2, (size_t)nb * nch);
  DA(f.ts, (size_t)nb * p->gulp * 4);
  DA(f.hts, (size_t)nb * p->gulp * 2);
  DA(b->d_dd, dd_floats * 4);
  DA(b->d_boxes, per_width * b->nwp);
  const size_t rw = (size_t)b->nrows * b->nbox;
  DA(b->d_rowmean, rw * 4);
  DA(b->d_rowmax, rw * 4);
  DA(b->d_rowvar, rw * 4);
  DA(b->d_counts, rw * 4);
  DA(b->d_offsets, rw * 4);
  DA(b->d_stats, (size_t)nb * b->nbox * 16);
  DA(b->d_gate, (size_t)nb * 16);
  DA(b->d_total, (size_t)nb * 4);
  DA(b->d_active, (size_t)nb * 4);
  DA(b->d_row_beam, (size_t)b->nrows * 4);
  DA(b->d_err, 16);
  DA(b->d_ntime, (size_t)nb * 4);
  DA(b->d_min_gulp, (size_t)nb * 4);
  DA(b->d_cand_i, (size_t)nb * cap * 16);
  DA(b->d_cand_v, (size_t)nb * cap * 4);
  DA(b->d_out, (size_t)nb * cap * sizeof(hella_cand));
  DA(b->d_dbeams, (size_t)nb * sizeof(hg::DedispBeam));
  DA(b->d_sbeams, (size_t)nb * sizeof(hg::SmoothBeam));
  DA(b->d_pos, sizeof(hg::GulpPos));
#undef DA
  if (cudaMallocHost((void **)&b->h_total, (size_t)nb * 4) != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_ALLOC);
  }
  b->hallocs.push_back(b->h_total);

  // host tables
  std::vector<uint8_t> keep((size_t)nb * nch, 1);
  if (bp->killmask)
    for (size_t i = 0; i < keep.size(); ++i) keep[i] = bp->killmask[i] != 0;
  std::vector<int> row_beam(b->nrows);
  std::vector<hg::SmoothBeam> sb(nb);
  b->dbeams.resize(nb);
  size_t dd_off = 0, box_off = 0;
  for (int i = 0; i < nb; ++i) {
    const int h = b->ndms[i] - 2;
    for (int r = 0; r < h; ++r) row_beam[row0[i] + r] = i;
    hg::DedispBeam &d = b->dbeams[i];
    d.packed = b->d_packed + (size_t)i * nch * R;
    d.out = b->d_dd + dd_off;
    d.win0 = 0;
    d.dm_count = b->ndms[i];
    d.item0 = 0;
    hg::SmoothBeam &B = sb[i];
    B.dd = b->d_dd + dd_off;
    B.dd_stride = b->ntime_dd;
    B.boxes = b->d_boxes + box_off;
    const size_t ro = (size_t)row0[i] * b->nbox;
    B.rowmean = b->d_rowmean + ro;
    B.rowmax = b->d_rowmax + ro;
    B.rowvar = b->d_rowvar + ro;
    B.counts = b->d_counts + ro;
    B.offsets = b->d_offsets + ro;
    B.stats = b->d_stats + (size_t)i * b->nbox * 4;
    B.gate = b->d_gate + (size_t)i * 4;
    B.cand_i = b->d_cand_i + (size_t)i * cap;
    B.cand_v = b->d_cand_v + (size_t)i * cap;
    B.total = b->d_total + i;
    B.active = b->d_active + i;
    B.h = h;
    B.row0 = row0[i];
    B.cap = (int)cap;
    B.beam_id = i + p->beam0;
    dd_off += (size_t)b->ndms[i] * b->ntime_dd;
    box_off += (size_t)b->nwp * h * b->ntime_out;
  }
  std::vector<float> taps;
  std::vector<int> toff, tn;
  hg::smoothing_taps(*p, b->nbox, &taps, &toff, &tn);
  if ((s = dalloc(b, (void **)&b->d_taps, taps.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(b, (void **)&b->d_tapoff, toff.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(b, (void **)&b->d_tapn, tn.size() * 4)) != HELLA_OK) return fail(s);
  const hg::GulpPos pos0{0, 0, 0, 0};
  if (cudaMemcpy(b->d_taps, taps.data(), taps.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_tapoff, toff.data(), toff.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_tapn, tn.data(), tn.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_keep, keep.data(), keep.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_row_beam, row_beam.data(), row_beam.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_sbeams, sb.data(), sb.size() * sizeof(hg::SmoothBeam), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->d_dbeams, b->dbeams.data(), nb * sizeof(hg::DedispBeam), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->d_ntime, b->ntime.data(), nb * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_min_gulp, b->min_gulp.data(), nb * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_pos, &pos0, sizeof(pos0), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(b->d_plain, 0, (size_t)nb * nch * R) != cudaSuccess ||
      cudaMemset(b->d_packed, 0, (size_t)nb * nch * R * 4) != cudaSuccess ||
      cudaMemset(b->d_err, 0, 16) != cudaSuccess || cudaMemset(b->d_total, 0, (size_t)nb * 4) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_CUDA);
  }
  if (p->autotune && (s = autotune(b, 2, nullptr, nullptr)) != HELLA_OK) return fail(s);
  *out = b;
  return HELLA_OK;
}

hella_status hella_batch_set_stream(hella_batch *b, void *stream) {
  if (!b) return HELLA_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(b->stream));
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;  // NULL: the batch's own stream
  hdd_set_stream(b->plan, b->stream);
  b->graph_stale = true;
  return HELLA_OK;
}

hella_status hella_batch_get_info(const hella_batch *b, int beam, hella_info *i) {
  if (!b || !i || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  i->ntime = b->ntime[beam];
  i->ndms = b->ndms[beam];
  i->max_delay = b->max_delay[beam];
  i->ntime_dd = b->ntime_dd;
  i->ntime_out = b->ntime_out;
  i->nboxcar = b->nbox;
  i->min_gulp = b->min_gulp[beam];
  i->gulp_index = b->gulp_index;
  i->device_bytes = b->dev_bytes;
  return HELLA_OK;
}

hella_status hella_batch_process_gulp(hella_batch *b, const uint8_t *gulp, int on_device,
                                      hella_cand *out, int max, int *n, int *counts, int *searched) {
  if (!b || !gulp || max < 0 || (max > 0 && !out)) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(b->p.device));
  const size_t bytes = (size_t)b->nbeam * b->p.gulp * b->p.nchan;
  CK(cudaMemcpyAsync(b->d_gulp, gulp, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     b->stream));
  hg::DedispArgs da;
  hella_status s = dedisp_args(b, b->tune, &da);
  if (s != HELLA_OK) return s;
  CK(cudaEventRecord(b->ev0, b->stream));
  if (b->use_graph) {
    if (b->graph_stale && (s = build_graph(b, da)) != HELLA_OK) return s;
    CK(cudaGraphLaunch(b->exec, b->stream));
  } else if ((s = enqueue_gulp(b, da)) != HELLA_OK) {
    return s;
  }
  CK(cudaEventRecord(b->ev1, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  int err = 0;
  CK(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(b->d_err, 0, sizeof(int));
    return HELLA_ERR_TIMEOUT;
  }
  long total = 0;
  for (int i = 0; i < b->nbeam; ++i) {
    total += b->h_total[i];
    if (counts) counts[i] = b->h_total[i];
    if (searched) searched[i] = b->gulp_index >= b->min_gulp[i];
  }
  const int k = (int)std::min<long>(total, max);
  if (k > 0)
    CK(cudaMemcpy(out, b->d_out, (size_t)k * sizeof(hella_cand), cudaMemcpyDeviceToHost));
  if (n) *n = k;
  b->gulp_index++;
  return HELLA_OK;
}

hella_status hella_batch_copy_dedisp(hella_batch *b, int beam, float *out) {
  if (!b || !out || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(out, b->dbeams[beam].out, (size_t)b->ndms[beam] * b->ntime_dd * 4, cudaMemcpyDeviceToHost));
  return HELLA_OK;
}

hella_status hella_batch_get_tuning(const hella_batch *b, hella_tuning *t) {
  if (!b || !t) return HELLA_ERR_INVALID_ARG;
  *t = b->tune;
  return HELLA_OK;
}

hella_status hella_batch_set_tuning(hella_batch *b, const hella_tuning *t) {
  if (!b || !t || !hg::tuning_ok(*t)) return HELLA_ERR_INVALID_ARG;
  b->tune = *t;
  b->tune.samples_per_thread = 4;
  b->graph_stale = true;
  return HELLA_OK;
}

hella_status hella_batch_time_dedisp(hella_batch *b, const hella_tuning *t, int reps, float *ms) {
  if (!b || !ms || reps < 1) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(b->p.device));
  return time_shape(b, t ? *t : b->tune, reps, ms);
}

hella_status hella_batch_autotune(hella_batch *b, int reps, hella_tuning *best, float *best_ms) {
  if (!b || reps < 1) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(b->p.device));
  return autotune(b, reps, best, best_ms);
}

hella_status hella_batch_graph_kernels(const hella_batch *b, int *kernels) {
  if (!b || !kernels) return HELLA_ERR_INVALID_ARG;
  *kernels = 0;
  if (!b->graph) return HELLA_ERR_STATE;
  size_t n = 0;
  CK(cudaGraphGetNodes(b->graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  CK(cudaGraphGetNodes(b->graph, nodes.data(), &n));
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    CK(cudaGraphNodeGetType(nd, &t));
    *kernels += t == cudaGraphNodeTypeKernel;
  }
  return HELLA_OK;
}

hella_status hella_batch_last_gulp_ms(const hella_batch *b, float *ms) {
  if (!b || !ms) return HELLA_ERR_INVALID_ARG;
  *ms = b->last_ms;
  return HELLA_OK;
}

}  // extern "C"
