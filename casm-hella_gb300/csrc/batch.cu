// batch.cu -- the batched multi-beam search and its streaming form
// (hella_batch_*, include/hella_search.h).
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
// trial up to the ceiling), so the plan's dedispersion tables serve every
// beam, each beam computing its own number of trials.  A beam that kills
// channels gets tables of its own over its unkilled channels (the same tile
// shape), so it sums only those; its killed channels are packed as zeros
// as well.
//
// Streaming.  Beams are slots: a dynamic batch sizes every slot for the
// largest DM list, and slots join and leave between gulps (the layout of
// rows and work items is rebuilt, the graph recaptured).  Up to two gulps
// are in flight, each with its own input and candidate buffers ("lanes"):
// the copy of gulp k+1 to the device runs on a copy stream while gulp k is
// searched.
#include "hella_dedisp.h"
#include "hella_search.h"
#include "hg_internal.h"
#include "hg_plan.h"
#include "hg_search.h"
#include "hg_tune.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

namespace {

// Ring positions and per-beam state of the gulp about to be processed.
__global__ void k_advance(hg::GulpPos *pos, hg::DedispBeam *db, int *active, int *total,
                          const int *ntime_b, const int *min_gulp_b, const int *member,
                          const int *join, int nbeam, long R, int gulp) {
  const long win0 = pos->win0;
  const int gi = pos->gulp_index;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) pos->wpos = (win0 + R - gulp) % R;
  if (b < nbeam) {
    db[b].win0 = (win0 + R - ntime_b[b]) % R;
    active[b] = member[b] && gi - join[b] >= min_gulp_b[b];  // casm_hella_refactored.cu:705
    total[b] = 0;
  }
}

// Running bandpass: ew += alpha * (bp - ew) per channel, the first gulp of a
// slot taking bp itself.  bp = calc_bandpass_new of the raw gulp.
__global__ void k_ew_bandpass(const float *bp, float *ew, const int *member, const int *join,
                              const hg::GulpPos *pos, int nbeam, int nchan, float alpha) {
  const int gi = pos->gulp_index;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (long)nbeam * nchan;
       i += (long)gridDim.x * blockDim.x) {
    const int b = (int)(i / nchan);
    if (!member[b]) continue;
    ew[i] = gi == join[b] ? bp[i] : __fadd_rn(ew[i], __fmul_rn(alpha, __fsub_rn(bp[i], ew[i])));
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

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// One gulp in flight: its input, candidate buffers, events and graph.
struct Lane {
  uint8_t *d_gulp = nullptr;
  hella_cand *d_out = nullptr;
  int *h_total = nullptr;
  cudaEvent_t copied = nullptr, t0 = nullptr, t1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool stale = true, busy = false;
  double submitted = 0;
  std::vector<int> searched;
};

// Sizes of a batch: DM lists per slot and the device bytes they imply.
struct Sizes {
  int ndms_all = 0, nbox = 0, ntime_dd = 0, ntime_out = 0;
  long R = 0;
  std::vector<int> cap_ndms;  // rows allocated per slot
  size_t fixed = 0, per_width = 0;
};

}  // namespace

struct hella_batch {
  hella_params p{};
  int nbeam = 0;
  bool dynamic = false, use_graph = true;
  float bp_alpha = 1.f;
  cudaStream_t stream = nullptr;  // graph capture needs a stream other than the legacy one
  cudaStream_t own_stream = nullptr, copy_stream = nullptr;
  hdd_plan plan = nullptr;        // the longest DM list; all channels active
  Sizes z;
  int nwp = 1, nrows = 0;
  std::vector<int> ndms, max_delay, ntime, min_gulp, member, join;
  std::vector<size_t> dd_off, box_off, row_off;
  int gulp_index = 0;             // gulps submitted
  size_t dev_bytes = 0;
  std::vector<void *> dallocs, hallocs;
  uint8_t *d_plain = nullptr, *d_keep = nullptr;
  uint32_t *d_packed = nullptr;
  hg::FlagState fs{};
  float *d_dd = nullptr, *d_boxes = nullptr, *d_taps = nullptr, *d_ew = nullptr;
  int *d_tapoff = nullptr, *d_tapn = nullptr;
  float *d_rowmean = nullptr, *d_rowmax = nullptr, *d_rowvar = nullptr, *d_stats = nullptr,
        *d_gate = nullptr;
  int *d_counts = nullptr, *d_offsets = nullptr, *d_total = nullptr, *d_active = nullptr,
      *d_row_beam = nullptr, *d_err = nullptr, *d_ntime = nullptr, *d_min_gulp = nullptr,
      *d_member = nullptr, *d_join = nullptr;
  int4 *d_cand_i = nullptr;
  float *d_cand_v = nullptr;
  hg::DedispBeam *d_dbeams = nullptr;
  hg::SmoothBeam *d_sbeams = nullptr;
  hg::GulpPos *d_pos = nullptr;
  std::vector<hg::DedispBeam> dbeams;
  int items_dpt = -1;             // DM tile of the work-item prefix held in d_dbeams
  std::vector<uint8_t> keep;      // [nbeam][nchan] killmasks (1: channel summed)
  int4 *d_bmeta = nullptr;        // per-beam tile tables (beams that kill channels)
  int *d_boff = nullptr, *d_bchans = nullptr;
  hg::TableJob *d_bjobs = nullptr;
  size_t bmeta_cap = 0, boff_cap = 0, bchans_cap = 0, bjobs_cap = 0;
  int btab_dpt = -1, btab_cc = -1;  // tile shape of the per-beam tables; -1: rebuild
  int *d_prend = nullptr;         // add modes 5, 6: [nbeam][npair] end of the rows each beam builds
  uint32_t *d_krows = nullptr;    // add modes 5, 6: rows of kbeams beams, krows_words apart
  long krows_words = 0;
  int kbeams = 0;
  int prend_key = -1;             // shape (groups per stage, channels per group) of d_prend; -1: remake
  hella_tuning tune{0, 4, 8, 0, hg::kDedispGroup, 0};
  std::vector<Lane> lanes;
  std::deque<int> queue;          // lanes in submission order
  int next_lane = 0;
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

hella_status halloc(hella_batch *b, void **ptr, size_t bytes) {
  if (cudaMallocHost(ptr, std::max<size_t>(bytes, 16)) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return HELLA_ERR_ALLOC;
  }
  b->hallocs.push_back(*ptr);
  return HELLA_OK;
}

// Number of trials of the DM list up to `ceiling`, which must be a prefix of
// the plan's list (-1 otherwise).
int prefix_trials(const hella_params &p, hdd_plan plan, float ceiling) {
  const std::vector<float> mine =
      hg::generate_dm_list((float)p.dm_min, ceiling, (float)p.ti_us, (float)p.dm_tol, p.nchan,
                           (float)p.plan_dt, (float)p.f0_mhz, (float)p.df_mhz);
  const int n = (int)hdd_get_dm_count(plan);
  if ((int)mine.size() > n) return -1;
  const float *all = hdd_get_dm_list(plan);
  for (size_t k = 0; k < mine.size(); ++k)
    if (mine[k] != all[k]) return -1;
  return (int)mine.size();
}

int ntime_of(const hella_params &p, int max_delay) {
  return 32 * ((p.gulp + max_delay + p.width_max) / 32 + 1);  // casm_hella_refactored.cu:217-219
}

// Plan and sizes of a batch (fixed slots: sized for their own ceilings;
// dynamic slots: for base.dm_max).
hella_status batch_sizes(const hella_batch_params *bp, hdd_plan *plan_out, Sizes *z) {
  const hella_params &p = bp->base;
  const int nb = p.nbeam, nch = p.nchan;
  float top = p.dm_max;
  if (bp->dm_max && !bp->dynamic) {
    top = bp->dm_max[0];
    for (int i = 0; i < nb; ++i) {
      if (!(bp->dm_max[i] >= p.dm_min)) return HELLA_ERR_INVALID_ARG;
      top = std::max(top, bp->dm_max[i]);
    }
  }
  hdd_plan plan = nullptr;
  if (hdd_create_plan(&plan, nch, (float)p.plan_dt, (float)p.f0_mhz, (float)p.df_mhz) != HDD_NO_ERROR ||
      hdd_generate_dm_list(plan, p.dm_min, top, p.ti_us, p.dm_tol) != HDD_NO_ERROR) {
    hdd_destroy_plan(plan);
    return HELLA_ERR_DEDISP;
  }
  z->ndms_all = (int)hdd_get_dm_count(plan);
  if (z->ndms_all < 3) {
    hdd_destroy_plan(plan);
    return HELLA_ERR_INVALID_ARG;
  }
  const int *delays = hdd_get_delay_table(plan);
  z->cap_ndms.assign(nb, z->ndms_all);
  z->R = 0;
  for (int i = 0; i < nb; ++i) {
    if (bp->dm_max && !bp->dynamic) {
      const int n = prefix_trials(p, plan, bp->dm_max[i]);
      if (n < 3) {
        hdd_destroy_plan(plan);
        return n < 0 ? HELLA_ERR_DEDISP : HELLA_ERR_INVALID_ARG;
      }
      z->cap_ndms[i] = n;
    }
    z->R = std::max<long>(z->R, ntime_of(p, delays[(size_t)(z->cap_ndms[i] - 1) * nch + nch - 1]));
  }
  z->ntime_dd = p.gulp + p.width_max;
  z->ntime_out = p.gulp;
  z->nbox = 0;
  for (int sm = p.width_min; sm < p.width_max; sm *= 2) z->nbox++;
  size_t dd_floats = 0, rows = 0, tab_bytes = 0;
  for (int i = 0; i < nb; ++i) {
    dd_floats += (size_t)z->cap_ndms[i] * z->ntime_dd;
    rows += (size_t)z->cap_ndms[i] - 2;
    // per-beam tile tables: 5-6 bytes per trial and channel (16- or 8-trial tiles)
    tab_bytes += (size_t)(z->cap_ndms[i] + 15) * nch * 6;
  }
  const size_t R = z->R, cap = p.max_giants;
  const size_t lanes = bp->inflight == 2 ? 2 : 1;
  z->fixed = lanes * hg::gulp_bytes(p) + (size_t)nb * nch * R * 5 + (size_t)nb * nch * 5 +
             (size_t)nb * nch * (256 * 6 + 16) + (size_t)nb * p.gulp * 6 + dd_floats * 4 + rows * z->nbox * 20 +
             (p.nscrunch > 0 || p.input_format ? (size_t)nb * nch * ((size_t)p.gulp * 6 + 8) : 0) +
             (size_t)nch * 4 +
             (size_t)nb * cap * 20 + lanes * (size_t)nb * cap * sizeof(hella_cand) + (size_t)nb * 512 +
             tab_bytes;
  z->per_width = rows * z->ntime_out * 4;
  *plan_out = plan;
  return HELLA_OK;
}

// Rows, smoothing table and dedispersion beams of the member slots, to the
// device; the next gulp recaptures its graph.
hella_status upload_layout(hella_batch *b) {
  const int nb = b->nbeam;
  const size_t cap = b->p.max_giants;
  std::vector<int> row_beam;
  std::vector<hg::SmoothBeam> sb(nb);
  b->nrows = 0;
  for (int i = 0; i < nb; ++i) {
    const int h = b->member[i] ? b->ndms[i] - 2 : 0;
    hg::SmoothBeam &B = sb[i];
    B.dd = b->d_dd + b->dd_off[i];
    B.dd_stride = b->z.ntime_dd;
    B.boxes = b->d_boxes + b->box_off[i];
    B.rowmean = b->d_rowmean + b->row_off[i];
    B.rowmax = b->d_rowmax + b->row_off[i];
    B.rowvar = b->d_rowvar + b->row_off[i];
    B.counts = b->d_counts + b->row_off[i];
    B.offsets = b->d_offsets + b->row_off[i];
    B.stats = b->d_stats + (size_t)i * b->z.nbox * 4;
    B.gate = b->d_gate + (size_t)i * 4;
    B.cand_i = b->d_cand_i + (size_t)i * cap;
    B.cand_v = b->d_cand_v + (size_t)i * cap;
    B.total = b->d_total + i;
    B.active = b->d_active + i;
    B.h = b->ndms[i] - 2;
    B.row0 = b->nrows;
    B.cap = (int)cap;
    B.beam_id = i + b->p.beam0;
    for (int r = 0; r < h; ++r) row_beam.push_back(i);
    b->nrows += h;
    hg::DedispBeam &d = b->dbeams[i];
    d.packed = b->d_packed + (size_t)i * b->p.nchan * b->z.R;
    d.out = b->d_dd + b->dd_off[i];
    d.win0 = 0;
    d.dm_count = b->member[i] ? b->ndms[i] : 0;
    d.item0 = 0;
  }
  CK(cudaStreamSynchronize(b->stream));
  if (!row_beam.empty())
    CK(cudaMemcpy(b->d_row_beam, row_beam.data(), row_beam.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_sbeams, sb.data(), sb.size() * sizeof(hg::SmoothBeam), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_ntime, b->ntime.data(), nb * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_min_gulp, b->min_gulp.data(), nb * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_member, b->member.data(), nb * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_join, b->join.data(), nb * 4, cudaMemcpyHostToDevice));
  b->items_dpt = -1;  // dedisp_args re-uploads the beams with their item prefix
  b->btab_dpt = -1;   // and rebuilds the per-beam tables
  b->prend_key = -1;  // and the per-beam row ends of add modes 5 and 6
  for (Lane &l : b->lanes) l.stale = true;
  return HELLA_OK;
}

// Slot i's sizes for `ndms` trials.
void set_slot_sizes(hella_batch *b, int i, int ndms) {
  const int nch = b->p.nchan;
  const int *delays = hdd_get_delay_table(b->plan);
  b->ndms[i] = ndms;
  b->max_delay[i] = delays[(size_t)(ndms - 1) * nch + nch - 1];
  b->ntime[i] = ntime_of(b->p, b->max_delay[i]);
  b->min_gulp[i] = b->ntime[i] / b->p.gulp;  // casm_hella_refactored.cu:632
}

// Regrows a device table buffer (its contents are rewritten after).
hella_status grow_table(void **ptr, size_t *cap, size_t need) {
  if (*cap >= need) return HELLA_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  if (cudaMalloc(ptr, need) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_ALLOC;
  }
  *cap = need;
  return HELLA_OK;
}

// Tile tables of their own for the member beams that kill channels: the
// rows of the plan's tables (all channels, same tile shape) of the beam's
// unkilled channels, so the tiles, delays and offsets are the plan's.
// Beams that keep every channel read the plan's tables.  Tiles of 1-4
// trials (very coarse DM lists) keep the plan's tables for every beam.
hella_status beam_tables(hella_batch *b, const hg::DeviceTables &tb) {
  const int nb = b->nbeam, nch = b->p.nchan;
  if (tb.nact != nch) return HELLA_ERR_DEDISP;  // the plan keeps every channel
  std::vector<hg::TableJob> jobs;
  std::vector<int> chans;
  std::vector<long> mo(nb, -1);
  std::vector<int> nact(nb, 0);
  long meta_n = 0;
  int max_tiles = 0;
  try {
    for (int i = 0; i < nb && tb.dpt >= 8; ++i) {
      if (!b->member[i]) continue;
      const int c0 = (int)chans.size();
      for (int c = 0; c < nch; ++c)
        if (b->keep[(size_t)i * nch + c]) chans.push_back(c);
      const int n = (int)chans.size() - c0;
      if (n == nch) {
        chans.resize(c0);
        continue;
      }
      const int ntiles = (b->ndms[i] + tb.dpt - 1) / tb.dpt;
      nact[i] = n;
      mo[i] = meta_n;
      jobs.push_back(hg::TableJob{meta_n, c0, n, ntiles});
      meta_n += (long)ntiles * n;
      max_tiles = std::max(max_tiles, ntiles);
    }
  } catch (const std::bad_alloc &) {
    return HELLA_ERR_ALLOC;
  }
  CK(cudaStreamSynchronize(b->stream));
  hella_status s;
  if ((s = grow_table((void **)&b->d_bmeta, &b->bmeta_cap, std::max<size_t>(meta_n, 1) * sizeof(int4))) !=
          HELLA_OK ||
      (s = grow_table((void **)&b->d_boff, &b->boff_cap, std::max<size_t>(meta_n, 1) * tb.dpt * sizeof(int))) !=
          HELLA_OK ||
      (s = grow_table((void **)&b->d_bchans, &b->bchans_cap, std::max<size_t>(chans.size(), 1) * sizeof(int))) !=
          HELLA_OK ||
      (s = grow_table((void **)&b->d_bjobs, &b->bjobs_cap, std::max<size_t>(jobs.size(), 1) * sizeof(hg::TableJob))) !=
          HELLA_OK)
    return s;
  if (!jobs.empty()) {
    CK(cudaMemcpy(b->d_bchans, chans.data(), chans.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_bjobs, jobs.data(), jobs.size() * sizeof(hg::TableJob), cudaMemcpyHostToDevice));
    CK(hg::gather_tables(tb.meta, tb.off, nch, tb.dpt, b->d_bjobs, (int)jobs.size(), max_tiles, b->d_bchans,
                         b->d_bmeta, b->d_boff, b->stream));
    CK(cudaStreamSynchronize(b->stream));
  }
  for (int i = 0; i < nb; ++i) {
    hg::DedispBeam &d = b->dbeams[i];
    d.meta = mo[i] < 0 ? nullptr : b->d_bmeta + mo[i];
    d.off = mo[i] < 0 ? nullptr : b->d_boff + mo[i] * tb.dpt;
    d.nact = nact[i];
  }
  b->btab_dpt = tb.dpt;
  b->btab_cc = tb.cc;
  b->items_dpt = -1;  // the beams go to the device again
  return HELLA_OK;
}

// Frees the rows of add modes 5 and 6 (set up again on next use).
void release_krows(hella_batch *b) {
  if (b->d_krows) {
    cudaFree(b->d_krows);
    b->dev_bytes -= (size_t)b->kbeams * std::max<long>(b->krows_words, 4) * 4;
  }
  b->d_krows = nullptr;
  b->krows_words = 0;
  b->kbeams = 0;
}

// Dedispersion launch over all beams with tile shape t (tables uploaded).
hella_status dedisp_args(hella_batch *b, const hella_tuning &t, hg::DedispArgs *out) {
  if (!hg::tuning_ok(t)) return HELLA_ERR_INVALID_ARG;
  if (t.add_mode >= 5) {
    // rows of channel pairs (5) or quads (6) over every channel (killed channels are packed as zeros), built
    // and summed beam by beam in one row buffer; a beam builds the rows its
    // own trials use
    const int g = t.add_mode == 6 ? 4 : 2, cc = t.chan_chunk / 2, ntt = hg::dedisp_time_tiles(b->z.ntime_dd);
    if (b->p.hbm_budget) {
      size_t bytes = 0;
      if (hg::plan_pair_bytes(b->plan, 0, b->z.ndms_all, cc, ntt, g, &bytes) != HDD_NO_ERROR) return HELLA_ERR_DEDISP;
      if (b->dev_bytes + bytes + (size_t)b->nbeam * b->p.nchan * 2 > b->p.hbm_budget) return HELLA_ERR_BUDGET;
    }
    hg::PairDeviceTables pt;
    const hdd_error he = hg::plan_pair_tables(b->plan, 0, b->z.ndms_all, cc, ntt, g, &pt, false);
    if (he == HDD_MEM_ALLOC_FAILED) return HELLA_ERR_ALLOC;
    if (he != HDD_NO_ERROR || pt.nact != b->p.nchan) return HELLA_ERR_DEDISP;  // the plan keeps every channel
    hella_status s;
    if (b->krows_words != pt.words) {  // rows of up to kPairMaxBeams beams, as many as memory and budget allow
      release_krows(b);
      const size_t per = (size_t)std::max<long>(pt.words, 4) * 4;
      for (int k = hg::kPairMaxBeams; k >= 1 && !b->d_krows; k /= 2) {
        if (b->p.hbm_budget && b->dev_bytes + k * per > b->p.hbm_budget) continue;
        if (cudaMalloc((void **)&b->d_krows, k * per) != cudaSuccess) {
          cudaGetLastError();
          b->d_krows = nullptr;
          continue;
        }
        b->kbeams = k;
        b->dev_bytes += k * per;
      }
      if (!b->d_krows) return b->p.hbm_budget ? HELLA_ERR_BUDGET : HELLA_ERR_ALLOC;
      b->krows_words = pt.words;
    }
    pt.rows = b->d_krows;
    if (!b->d_prend && (s = dalloc(b, (void **)&b->d_prend, (size_t)b->nbeam * pt.npair * 4)) != HELLA_OK)
      return s;
    if (b->prend_key != cc * 16 + g) {
      std::vector<int> ends((size_t)b->nbeam * pt.npair);
      for (int i = 0; i < b->nbeam; ++i)
        if (hg::plan_pair_row_ends(b->plan, b->dbeams[i].dm_count, &ends[(size_t)i * pt.npair]) != HDD_NO_ERROR)
          return HELLA_ERR_DEDISP;
      CK(cudaStreamSynchronize(b->stream));
      CK(cudaMemcpy(b->d_prend, ends.data(), ends.size() * 4, cudaMemcpyHostToDevice));
      b->prend_key = cc * 16 + g;
    }
    hg::DedispArgs a{};
    a.nbeam = 1;
    a.ntt = ntt;
    int items = 0;
    for (int i = 0; i < b->nbeam; ++i) {
      b->dbeams[i].item0 = items;
      items += hg::dedisp_items(b->dbeams[i].dm_count, hg::kPairDPT, ntt);
    }
    if (b->items_dpt != hg::kPairDPT) {
      CK(cudaStreamSynchronize(b->stream));
      CK(cudaMemcpy(b->d_dbeams, b->dbeams.data(), sizeof(hg::DedispBeam) * b->nbeam, cudaMemcpyHostToDevice));
      b->items_dpt = hg::kPairDPT;
    }
    a.nitems = items;
    a.group = t.group;
    a.R = b->z.R;
    a.dm_first = 0;
    a.nout = b->z.ntime_dd;
    a.out_stride = b->z.ntime_dd;
    a.nbuf = t.stages;
    a.unit = 1;
    a.err = b->d_err;
    hg::use_pair_tables(&a, pt);
    *out = a;
    return HELLA_OK;
  }
  if (t.add_mode == 4) {
    // sub-band sums over every channel: a beam's killed channels are packed
    // as zeros, so the plan's tables serve every beam
    hg::SubDeviceTables sb;
    if (hg::plan_sub_tables(b->plan, 0, b->z.ndms_all, &sb) != HDD_NO_ERROR) return HELLA_ERR_DEDISP;
    if (sb.nact != b->p.nchan) return HELLA_ERR_DEDISP;  // the plan keeps every channel
    hg::DedispArgs a{};
    a.beams = b->d_dbeams;
    a.nbeam = b->nbeam;
    a.ntt = hg::dedisp_time_tiles(b->z.ntime_dd);
    int items = 0;
    for (int i = 0; i < b->nbeam; ++i) {
      b->dbeams[i].item0 = items;
      items += hg::dedisp_items(b->dbeams[i].dm_count, hg::kSubDPT, a.ntt);
    }
    if (b->items_dpt != hg::kSubDPT) {
      CK(cudaStreamSynchronize(b->stream));
      CK(cudaMemcpy(b->d_dbeams, b->dbeams.data(), sizeof(hg::DedispBeam) * b->nbeam, cudaMemcpyHostToDevice));
      b->items_dpt = hg::kSubDPT;
    }
    a.nitems = items;
    a.group = t.group;
    a.R = b->z.R;
    a.dm_first = 0;
    a.nout = b->z.ntime_dd;
    a.out_stride = b->z.ntime_dd;
    a.cc = hg::kSubG;
    a.nbuf = t.stages;
    a.unit = 1;
    a.err = b->d_err;
    hg::use_sub_tables(&a, sb);
    *out = a;
    return HELLA_OK;
  }
  hg::DeviceTables tb;
  if (hg::plan_device_tables(b->plan, 0, b->z.ndms_all, &tb, t.dm_per_block, t.chan_chunk) != HDD_NO_ERROR)
    return HELLA_ERR_DEDISP;
  if (t.add_mode && tb.dpt < 8) return HELLA_ERR_INVALID_ARG;
  hella_status s;
  if ((b->btab_dpt != tb.dpt || b->btab_cc != tb.cc) && (s = beam_tables(b, tb)) != HELLA_OK) return s;
  hg::DedispArgs a{};
  a.beams = b->d_dbeams;
  a.nbeam = b->nbeam;
  a.ntt = hg::dedisp_time_tiles(b->z.ntime_dd);
  // work-item prefix of this DM tile (win0 is rewritten on the device each gulp)
  int items = 0;
  for (int i = 0; i < b->nbeam; ++i) {
    b->dbeams[i].item0 = items;
    items += hg::dedisp_items(b->dbeams[i].dm_count, tb.dpt, a.ntt);
  }
  if (b->items_dpt != tb.dpt) {
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaMemcpy(b->d_dbeams, b->dbeams.data(), sizeof(hg::DedispBeam) * b->nbeam, cudaMemcpyHostToDevice));
    b->items_dpt = tb.dpt;
  }
  a.nitems = items;
  a.group = t.group;
  a.R = b->z.R;
  a.nact = tb.nact;
  a.dm_first = 0;
  a.nout = b->z.ntime_dd;
  a.out_stride = b->z.ntime_dd;
  a.dpt = tb.dpt;
  a.cc = tb.cc;
  a.nbuf = t.stages;
  a.mode = t.add_mode;
  a.unit = 1;
  a.max_spread = tb.max_spread;
  a.tile_meta = tb.meta;
  a.tile_off = tb.off;
  a.err = b->d_err;
  for (int i = 0; i < b->nbeam; ++i) a.varied |= b->dbeams[i].meta != nullptr;
  *out = a;
  return HELLA_OK;
}

// The dedispersion of every beam: one persistent launch, or (add modes 5, 6)
// the rows built and summed beam by beam, each launch reading its beam's
// ring position from the device.
hella_status dedisperse_beams(hella_batch *b, const hg::DedispArgs &da) {
  if (da.mode < 5) {
    CK(hg::dedisperse(da, b->stream));
    return HELLA_OK;
  }
  for (int i = 0; i < b->nbeam; i += b->kbeams) {  // kbeams beams a build and a sum launch
    const int nk = std::min(b->kbeams, b->nbeam - i);
    int items = 0;
    for (int z = 0; z < nk; ++z) items += hg::dedisp_items(b->dbeams[i + z].dm_count, hg::kPairDPT, da.ntt);
    if (items == 0) continue;
    hg::DedispArgs a = da;
    a.beams = b->d_dbeams + i;
    a.nbeam = nk;
    a.one = b->dbeams[i];
    a.nitems = items;
    a.pair_rend = b->d_prend + (size_t)i * da.pair_npair;
    const cudaError_t e = hg::dedisperse(a, b->stream);
    if (e == cudaErrorInvalidValue) {  // the DM list's stages do not fit this kernel's staging
      cudaGetLastError();
      return HELLA_ERR_INVALID_ARG;
    }
    CK(e);
  }
  return HELLA_OK;
}

hg::SmoothArgs smooth_args(hella_batch *b, int w0, int nw) {
  hg::SmoothArgs a{};
  a.beams = b->d_sbeams;
  a.nbeam = b->nbeam;
  a.row_beam = b->d_row_beam;
  a.nrows = b->nrows;
  a.ntime_dd = b->z.ntime_dd;
  a.ntime_out = b->z.ntime_out;
  a.nbox = b->z.nbox;
  a.wmin = b->p.width_min;
  a.wmax = b->p.width_max;
  a.anchor = b->p.smooth_anchor;
  a.w0 = w0;
  a.nw = nw;
  a.taps = b->d_taps;
  a.tap_off = b->d_tapoff;
  a.tap_n = b->d_tapn;
  a.snr = b->p.snr;
  a.nogate = b->p.always_find_peaks != 0;
  return a;
}

// Every launch of one gulp, in order, on b->stream (captured or not).
hella_status enqueue_gulp(hella_batch *b, const hg::DedispArgs &da, Lane &l) {
  const int nb = b->nbeam, nch = b->p.nchan;
  k_advance<<<(nb + 255) / 256, 256, 0, b->stream>>>(b->d_pos, b->d_dbeams, b->d_active, b->d_total,
                                                     b->d_ntime, b->d_min_gulp, b->d_member, b->d_join, nb,
                                                     b->z.R, b->p.gulp);
  CK(hg::flag_gulp_dev(b->fs, l.d_gulp, b->d_plain, b->z.R, b->d_pos, b->stream));
  k_ew_bandpass<<<std::min(1024, (nb * nch + 255) / 256), 256, 0, b->stream>>>(
      b->fs.bp1, b->d_ew, b->d_member, b->d_join, b->d_pos, nb, nch, b->bp_alpha);
  CK(hg::pack_gulp_dev(b->d_plain, b->d_packed, nb, nch, b->z.R, b->p.gulp, b->d_pos, b->stream, b->d_keep));
  hella_status st;
  if (da.nitems > 0 && (st = dedisperse_beams(b, da)) != HELLA_OK) return st;
  for (int w0 = 0; w0 < b->z.nbox; w0 += b->nwp) {
    const hg::SmoothArgs a = smooth_args(b, w0, std::min(b->nwp, b->z.nbox - w0));
    CK(hg::smooth_planes(a, b->stream));
    CK(hg::smooth_stats(a, b->stream, 1));
    CK(hg::find_peaks(a, b->stream));
  }
  k_gather<<<nb, 256, 0, b->stream>>>(b->d_sbeams, b->d_total, nb, l.d_out);
  CK(cudaMemcpyAsync(l.h_total, b->d_total, sizeof(int) * nb, cudaMemcpyDeviceToHost, b->stream));
  k_rewind<<<1, 1, 0, b->stream>>>(b->d_pos, b->z.R, b->p.gulp);
  hg::count_launches(4);
  CK(cudaGetLastError());
  return HELLA_OK;
}

// Captures lane l's gulp sequence into its executable graph.
hella_status build_graph(hella_batch *b, const hg::DedispArgs &da, Lane &l) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const hella_status s = enqueue_gulp(b, da, l);
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (s != HELLA_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return s != HELLA_OK ? s : HELLA_ERR_CUDA;
  }
  if (l.exec) cudaGraphExecDestroy(l.exec);
  if (l.graph) cudaGraphDestroy(l.graph);
  l.exec = nullptr;
  l.graph = g;
  if (cudaGraphInstantiate(&l.exec, g, 0) != cudaSuccess) {
    cudaGetLastError();
    l.exec = nullptr;
    return HELLA_ERR_CUDA;
  }
  l.stale = false;
  return HELLA_OK;
}

hella_status time_shape(hella_batch *b, const hella_tuning &t, int reps, float *ms) {
  hg::DedispArgs da;
  hella_status s = dedisp_args(b, t, &da);
  if (s != HELLA_OK) return s;
  if (da.nitems == 0) return HELLA_ERR_STATE;
  s = hg::time_runs(b->stream, reps, [&]() -> hella_status { return dedisperse_beams(b, da); }, ms);
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
  if (best.add_mode < 5) {  // the rows are only kept for add modes 5 and 6
    hg::plan_pair_release(b->plan);
    release_krows(b);
  }
  for (Lane &l : b->lanes) l.stale = true;
  if (out) *out = best;
  if (out_ms) *out_ms = best_ms;
  return HELLA_OK;
}

bool any_busy(const hella_batch *b) {
  for (const Lane &l : b->lanes)
    if (l.busy) return true;
  return false;
}

}  // namespace

extern "C" {

void hella_batch_params_default(hella_batch_params *p) {
  std::memset(p, 0, sizeof(*p));
  hella_params_default(&p->base);
  p->use_graph = 1;
  p->inflight = 1;
  p->bp_alpha = 0.1f;
}

void hella_batch_destroy(hella_batch *b) {
  if (!b) return;
  cudaSetDevice(b->p.device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->copy_stream) cudaStreamSynchronize(b->copy_stream);
  for (Lane &l : b->lanes) {
    if (l.exec) cudaGraphExecDestroy(l.exec);
    if (l.graph) cudaGraphDestroy(l.graph);
    if (l.copied) cudaEventDestroy(l.copied);
    if (l.t0) cudaEventDestroy(l.t0);
    if (l.t1) cudaEventDestroy(l.t1);
  }
  for (void *ptr : b->dallocs) cudaFree(ptr);
  for (void *ptr : b->hallocs) cudaFreeHost(ptr);
  for (void *ptr : {(void *)b->d_bmeta, (void *)b->d_boff, (void *)b->d_bchans, (void *)b->d_bjobs,
                    (void *)b->d_krows})
    if (ptr) cudaFree(ptr);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
  hdd_destroy_plan(b->plan);
  delete b;
}

hella_status hella_batch_bytes(const hella_batch_params *bp, size_t *bytes) {
  if (!bp || !bytes) return HELLA_ERR_INVALID_ARG;
  hella_status s = hg::validate_params(&bp->base);
  if (s != HELLA_OK) return s;
  hdd_plan plan = nullptr;
  Sizes z;
  if ((s = batch_sizes(bp, &plan, &z)) != HELLA_OK) return s;
  hdd_destroy_plan(plan);
  const int nw = bp->widths_per_pass ? std::min(bp->widths_per_pass, z.nbox) : z.nbox;
  *bytes = z.fixed + z.per_width * nw;
  return HELLA_OK;
}

hella_status hella_batch_create(hella_batch **out, const hella_batch_params *bp) {
  if (!out || !bp) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  const hella_params *p = &bp->base;
  hella_status s = hg::validate_params(p);
  if (s != HELLA_OK) return s;
  if (bp->widths_per_pass < 0 || (bp->inflight != 1 && bp->inflight != 2) || !(bp->bp_alpha > 0.f) ||
      bp->bp_alpha > 1.f)
    return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(p->device) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  hella_batch *b = new (std::nothrow) hella_batch;
  if (!b) return HELLA_ERR_ALLOC;
  b->p = *p;
  b->nbeam = p->nbeam;
  b->use_graph = bp->use_graph != 0;
  b->dynamic = bp->dynamic != 0;
  b->bp_alpha = bp->bp_alpha;
  auto fail = [&](hella_status st) {
    hella_batch_destroy(b);
    return st;
  };
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_CUDA);
  }
  b->stream = b->own_stream;
  const int nb = b->nbeam, nch = p->nchan;
  if ((s = batch_sizes(bp, &b->plan, &b->z)) != HELLA_OK) return fail(s);
  const Sizes &z = b->z;

  // slots: DM ceilings (dynamic slots take base.dm_max unless dm_max says otherwise)
  b->ndms.resize(nb);
  b->max_delay.resize(nb);
  b->ntime.resize(nb);
  b->min_gulp.resize(nb);
  b->member.assign(nb, 1);
  b->join.assign(nb, 0);
  if (bp->member)
    for (int i = 0; i < nb; ++i) b->member[i] = bp->member[i] != 0;
  for (int i = 0; i < nb; ++i) {
    int n = z.cap_ndms[i];
    if (b->dynamic && bp->dm_max) {
      if (bp->dm_max[i] > p->dm_max) return fail(HELLA_ERR_BUDGET);
      n = prefix_trials(*p, b->plan, bp->dm_max[i]);
      if (n < 3) return fail(n < 0 ? HELLA_ERR_DEDISP : HELLA_ERR_INVALID_ARG);
    }
    set_slot_sizes(b, i, n);
  }

  // HBM: everything but the smoothed planes, then as many widths per pass
  // as the budget allows
  size_t budget = p->hbm_budget;
  if (!budget) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return fail(HELLA_ERR_CUDA);
    budget = fr > (1ul << 30) ? fr - (1ul << 30) : 0;  // leave 1 GB to the runtime
  }
  if (z.fixed + z.per_width > budget) return fail(HELLA_ERR_BUDGET);
  b->nwp = bp->widths_per_pass ? std::min(bp->widths_per_pass, z.nbox)
                               : (int)std::min<size_t>(z.nbox, (budget - z.fixed) / z.per_width);
  if (b->nwp < 1 || z.fixed + z.per_width * b->nwp > budget) return fail(HELLA_ERR_BUDGET);

  const size_t R = z.R, cap = p->max_giants;
  size_t dd_floats = 0, rows = 0;
  b->dd_off.resize(nb);
  b->box_off.resize(nb);
  b->row_off.resize(nb);
  for (int i = 0; i < nb; ++i) {
    b->dd_off[i] = dd_floats;
    b->box_off[i] = rows * b->nwp * z.ntime_out;
    b->row_off[i] = rows * z.nbox;
    dd_floats += (size_t)z.cap_ndms[i] * z.ntime_dd;
    rows += (size_t)z.cap_ndms[i] - 2;
  }
#define DA(ptr, bytes)                                                  \
  if ((s = dalloc(b, (void **)&(ptr), (bytes))) != HELLA_OK) return fail(s);
  b->lanes.resize(bp->inflight);
  for (Lane &l : b->lanes) {
    DA(l.d_gulp, hg::gulp_bytes(*p));
    DA(l.d_out, (size_t)nb * cap * sizeof(hella_cand));
    if ((s = halloc(b, (void **)&l.h_total, (size_t)nb * 4)) != HELLA_OK) return fail(s);
    if (cudaEventCreate(&l.copied) != cudaSuccess || cudaEventCreate(&l.t0) != cudaSuccess ||
        cudaEventCreate(&l.t1) != cudaSuccess) {
      cudaGetLastError();
      return fail(HELLA_ERR_CUDA);
    }
  }
  DA(b->d_plain, (size_t)nb * nch * R);
  DA(b->d_packed, (size_t)nb * nch * R * 4);
  DA(b->d_keep, (size_t)nb * nch);
  DA(b->d_ew, (size_t)nb * nch * 4);
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
  hg::flag_scrunch_params(*p, &f);
  if (p->nscrunch > 0 || f.f16_input) {
    DA(f.P, (size_t)nb * nch * p->gulp * 2);
    DA(f.M, (size_t)nb * nch * p->gulp * 2);
    DA(f.S, (size_t)nb * nch * p->gulp * 2);
    DA(f.bpx, (size_t)nb * nch * 4);
    DA(f.fsb, (size_t)nb * nch * 4);
  }
  DA(f.flagspec, (size_t)nch * 4);
  DA(b->d_dd, dd_floats * 4);
  DA(b->d_boxes, z.per_width * b->nwp);
  const size_t rw = rows * z.nbox;
  DA(b->d_rowmean, rw * 4);
  DA(b->d_rowmax, rw * 4);
  DA(b->d_rowvar, rw * 4);
  DA(b->d_counts, rw * 4);
  DA(b->d_offsets, rw * 4);
  DA(b->d_stats, (size_t)nb * z.nbox * 16);
  DA(b->d_gate, (size_t)nb * 16);
  DA(b->d_total, (size_t)nb * 4);
  DA(b->d_active, (size_t)nb * 4);
  DA(b->d_row_beam, rows * 4);
  DA(b->d_err, 16);
  DA(b->d_ntime, (size_t)nb * 4);
  DA(b->d_min_gulp, (size_t)nb * 4);
  DA(b->d_member, (size_t)nb * 4);
  DA(b->d_join, (size_t)nb * 4);
  DA(b->d_cand_i, (size_t)nb * cap * 16);
  DA(b->d_cand_v, (size_t)nb * cap * 4);
  DA(b->d_dbeams, (size_t)nb * sizeof(hg::DedispBeam));
  DA(b->d_sbeams, (size_t)nb * sizeof(hg::SmoothBeam));
  DA(b->d_pos, sizeof(hg::GulpPos));
#undef DA

  b->keep.assign((size_t)nb * nch, 1);
  if (bp->killmask)
    for (size_t i = 0; i < b->keep.size(); ++i) b->keep[i] = bp->killmask[i] != 0;
  const std::vector<uint8_t> &keep = b->keep;
  b->dbeams.assign(nb, hg::DedispBeam{});
  std::vector<float> taps;
  std::vector<int> toff, tn;
  hg::smoothing_taps(*p, z.nbox, &taps, &toff, &tn);
  if ((s = dalloc(b, (void **)&b->d_taps, taps.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(b, (void **)&b->d_tapoff, toff.size() * 4)) != HELLA_OK) return fail(s);
  if ((s = dalloc(b, (void **)&b->d_tapn, tn.size() * 4)) != HELLA_OK) return fail(s);
  const hg::GulpPos pos0{0, 0, 0, 0};
  if (cudaMemcpy(b->d_taps, taps.data(), taps.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_tapoff, toff.data(), toff.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_tapn, tn.data(), tn.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_keep, keep.data(), keep.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_pos, &pos0, sizeof(pos0), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(b->d_plain, 0, (size_t)nb * nch * R) != cudaSuccess ||
      cudaMemset(b->d_packed, 0, (size_t)nb * nch * R * 4) != cudaSuccess ||
      cudaMemset(b->d_ew, 0, (size_t)nb * nch * 4) != cudaSuccess ||
      cudaMemset(f.flagspec, 0, (size_t)nch * 4) != cudaSuccess ||
      cudaMemset(b->d_err, 0, 16) != cudaSuccess || cudaMemset(b->d_total, 0, (size_t)nb * 4) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    return fail(HELLA_ERR_CUDA);
  }
  if ((s = upload_layout(b)) != HELLA_OK) return fail(s);
  if (p->autotune && b->nrows > 0 && (s = autotune(b, 2, nullptr, nullptr)) != HELLA_OK) return fail(s);
  *out = b;
  return HELLA_OK;
}

hella_status hella_batch_set_stream(hella_batch *b, void *stream) {
  if (!b) return HELLA_ERR_INVALID_ARG;
  if (any_busy(b)) return HELLA_ERR_STATE;
  CK(cudaStreamSynchronize(b->stream));
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;  // NULL: the batch's own stream
  hdd_set_stream(b->plan, b->stream);
  for (Lane &l : b->lanes) l.stale = true;
  return HELLA_OK;
}

hella_status hella_batch_get_info(const hella_batch *b, int beam, hella_info *i) {
  if (!b || !i || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  i->ntime = b->ntime[beam];
  i->ndms = b->ndms[beam];
  i->max_delay = b->max_delay[beam];
  i->ntime_dd = b->z.ntime_dd;
  i->ntime_out = b->z.ntime_out;
  i->nboxcar = b->z.nbox;
  i->min_gulp = b->min_gulp[beam];
  i->gulp_index = b->gulp_index - b->join[beam];
  i->device_bytes = b->dev_bytes;
  return HELLA_OK;
}

hella_status hella_batch_set_beam(hella_batch *b, int beam, int member, float dm_max, const int *killmask) {
  if (!b || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  if (!b->dynamic || any_busy(b)) return HELLA_ERR_STATE;
  CK(cudaSetDevice(b->p.device));
  const int nch = b->p.nchan;
  if (member) {
    if (dm_max > b->p.dm_max) return HELLA_ERR_BUDGET;
    const int n = prefix_trials(b->p, b->plan, dm_max);
    if (n < 3) return n < 0 ? HELLA_ERR_DEDISP : HELLA_ERR_INVALID_ARG;
    set_slot_sizes(b, beam, n);
    uint8_t *keep = b->keep.data() + (size_t)beam * nch;
    for (int c = 0; c < nch; ++c) keep[c] = killmask ? killmask[c] != 0 : 1;
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaMemcpy(b->d_keep + (size_t)beam * nch, keep, nch, cudaMemcpyHostToDevice));
    // a fresh ring for the newcomer, as a new single-beam context starts with
    CK(cudaMemset(b->d_plain + (size_t)beam * nch * b->z.R, 0, (size_t)nch * b->z.R));
    CK(cudaMemset(b->d_packed + (size_t)beam * nch * b->z.R, 0, (size_t)nch * b->z.R * 4));
    b->join[beam] = b->gulp_index;
  }
  b->member[beam] = member != 0;
  return upload_layout(b);
}

hella_status hella_batch_get_flag_spec(hella_batch *b, float *out) {
  if (!b || !out) return HELLA_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(out, b->fs.flagspec, (size_t)b->p.nchan * 4, cudaMemcpyDeviceToHost));
  return HELLA_OK;
}

hella_status hella_batch_get_bandpass(hella_batch *b, int beam, float *out) {
  if (!b || !out || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(out, b->d_ew + (size_t)beam * b->p.nchan, (size_t)b->p.nchan * 4, cudaMemcpyDeviceToHost));
  return HELLA_OK;
}

hella_status hella_batch_submit(hella_batch *b, const uint8_t *gulp, int on_device) {
  if (!b || !gulp) return HELLA_ERR_INVALID_ARG;
  CK(cudaSetDevice(b->p.device));
  Lane &l = b->lanes[b->next_lane];
  if (l.busy) return HELLA_ERR_STATE;
  hg::DedispArgs da;
  hella_status s = dedisp_args(b, b->tune, &da);
  if (s != HELLA_OK) return s;
  l.submitted = now_ms();
  // the input copy waits for the last search that read this lane's buffers
  CK(cudaStreamWaitEvent(b->copy_stream, l.t1, 0));
  const size_t bytes = hg::gulp_bytes(b->p);
  CK(cudaMemcpyAsync(l.d_gulp, gulp, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     b->copy_stream));
  CK(cudaEventRecord(l.copied, b->copy_stream));
  CK(cudaStreamWaitEvent(b->stream, l.copied, 0));
  CK(cudaEventRecord(l.t0, b->stream));
  if (b->use_graph) {
    if (l.stale && (s = build_graph(b, da, l)) != HELLA_OK) return s;
    CK(cudaGraphLaunch(l.exec, b->stream));
  } else if ((s = enqueue_gulp(b, da, l)) != HELLA_OK) {
    return s;
  }
  CK(cudaEventRecord(l.t1, b->stream));
  l.searched.resize(b->nbeam);
  for (int i = 0; i < b->nbeam; ++i)
    l.searched[i] = b->member[i] && b->gulp_index - b->join[i] >= b->min_gulp[i];
  l.busy = true;
  b->queue.push_back(b->next_lane);
  b->next_lane = (b->next_lane + 1) % (int)b->lanes.size();
  b->gulp_index++;
  return HELLA_OK;
}

hella_status hella_batch_poll(hella_batch *b, hella_cand *out, int max, int *n, int *counts, int *searched,
                              float *latency_ms, float *device_ms) {
  if (!b || max < 0 || (max > 0 && !out)) return HELLA_ERR_INVALID_ARG;
  if (b->queue.empty()) return HELLA_ERR_STATE;
  CK(cudaSetDevice(b->p.device));
  Lane &l = b->lanes[b->queue.front()];
  CK(cudaEventSynchronize(l.t1));
  b->queue.pop_front();
  l.busy = false;
  cudaEventElapsedTime(&b->last_ms, l.t0, l.t1);
  int err = 0;
  CK(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(b->d_err, 0, sizeof(int));
    return HELLA_ERR_TIMEOUT;
  }
  long total = 0;
  for (int i = 0; i < b->nbeam; ++i) {
    total += l.h_total[i];
    if (counts) counts[i] = l.h_total[i];
    if (searched) searched[i] = l.searched[i];
  }
  const int k = (int)std::min<long>(total, max);
  if (k > 0) CK(cudaMemcpy(out, l.d_out, (size_t)k * sizeof(hella_cand), cudaMemcpyDeviceToHost));
  if (n) *n = k;
  if (device_ms) *device_ms = b->last_ms;
  if (latency_ms) *latency_ms = (float)(now_ms() - l.submitted);
  return HELLA_OK;
}

hella_status hella_batch_process_gulp(hella_batch *b, const uint8_t *gulp, int on_device, hella_cand *out,
                                      int max, int *n, int *counts, int *searched) {
  if (!b || !gulp || max < 0 || (max > 0 && !out)) return HELLA_ERR_INVALID_ARG;
  if (!b->queue.empty()) return HELLA_ERR_STATE;
  hella_status s = hella_batch_submit(b, gulp, on_device);
  if (s != HELLA_OK) return s;
  return hella_batch_poll(b, out, max, n, counts, searched, nullptr, nullptr);
}

hella_status hella_batch_copy_dedisp(hella_batch *b, int beam, float *out) {
  if (!b || !out || beam < 0 || beam >= b->nbeam) return HELLA_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(out, b->d_dd + b->dd_off[beam], (size_t)b->ndms[beam] * b->z.ntime_dd * 4,
                cudaMemcpyDeviceToHost));
  return HELLA_OK;
}

hella_status hella_batch_get_tuning(const hella_batch *b, hella_tuning *t) {
  if (!b || !t) return HELLA_ERR_INVALID_ARG;
  *t = b->tune;
  return HELLA_OK;
}

hella_status hella_batch_set_tuning(hella_batch *b, const hella_tuning *t) {
  if (!b || !t || !hg::tuning_ok(*t)) return HELLA_ERR_INVALID_ARG;
  if (any_busy(b)) return HELLA_ERR_STATE;
  b->tune = *t;
  if (t->add_mode < 5) {
    hg::plan_pair_release(b->plan);
    release_krows(b);
  }
  b->tune.samples_per_thread = 4;
  for (Lane &l : b->lanes) l.stale = true;
  return HELLA_OK;
}

hella_status hella_batch_time_dedisp(hella_batch *b, const hella_tuning *t, int reps, float *ms) {
  if (!b || !ms || reps < 1) return HELLA_ERR_INVALID_ARG;
  if (any_busy(b)) return HELLA_ERR_STATE;
  CK(cudaSetDevice(b->p.device));
  return time_shape(b, t ? *t : b->tune, reps, ms);
}

hella_status hella_batch_autotune(hella_batch *b, int reps, hella_tuning *best, float *best_ms) {
  if (!b || reps < 1) return HELLA_ERR_INVALID_ARG;
  if (any_busy(b)) return HELLA_ERR_STATE;
  CK(cudaSetDevice(b->p.device));
  return autotune(b, reps, best, best_ms);
}

hella_status hella_batch_graph_kernels(const hella_batch *b, int *kernels) {
  if (!b || !kernels) return HELLA_ERR_INVALID_ARG;
  *kernels = 0;
  const cudaGraph_t g = b->lanes.empty() ? nullptr : b->lanes[0].graph;
  if (!g) return HELLA_ERR_STATE;
  size_t n = 0;
  CK(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  CK(cudaGraphGetNodes(g, nodes.data(), &n));
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
