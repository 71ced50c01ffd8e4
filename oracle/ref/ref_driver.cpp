/*
 * ref_driver.cpp -- calls into the reference's own stage code, built for
 * the CPU under emu_cuda.h, with the pinfo_t fields each stage reads set up
 * the way initialize() does (src/apps/casm_hella_refactored.cu:54-309).
 * TEST INFRASTRUCTURE ONLY: generates the golden fixtures that pin the
 * oracle (tests/golden/make_golden.py).
 */
#include "hella/alloc.h"
#include "hella/definitions.h"
#include "hella/flagger.h"
#include "hella/median_filter.h"
#include "hella/normalization.h"
#include "hella/peaks.h"
#include "hella/smooth.h"

#include <cstring>
#include <vector>

extern std::vector<float> g_taps_seen;

extern "C" {

int ref_nchan(void) { return NCHAN; }

/* fast_flagger (flagger.cu:345-411) on one beam: u8 [w][NCHAN] in, the
 * beam's u8 ring (NTIME = w, so the whole ring is this gulp) out, with the
 * time series and the accumulated flag spectrum. */
int ref_flag(const uint8_t *gulp, int w, float spec_min, float spec_max, int flag1, int flag2, int nscrunch,
             const int *tscr, const int *fscr, const float *thresh, uint8_t *out, float *ts, float *flagspec) {
  hella::pinfo_t p{};
  p.inp_format = 2;
  p.nbeam = 1;
  p.gulp = (unsigned long)w;
  p.NTIME = (unsigned long)w;
  p.spec_min = spec_min;
  p.spec_max = spec_max;
  p.flag1 = flag1;
  p.flag2 = flag2;
  p.nscrunches = nscrunch;
  std::vector<hella::scrunch> sc(nscrunch > 0 ? nscrunch : 1);
  for (int i = 0; i < nscrunch; ++i) {
    sc[i].tscrunch = tscr[i];
    sc[i].fscrunch = fscr[i];
    sc[i].thresh = thresh[i];
    sc[i].nits = 1;
  }
  p.scrunches = sc.data();
  p.gulp_nbyte = 1;
  hella::alloc_gpu<unsigned char>(&p.d_gulp, (size_t)w * NCHAN);
  std::memcpy(p.d_gulp, gulp, (size_t)w * NCHAN);
  hella::alloc_gpu<unsigned char>(&p.d_data, (size_t)w * NCHAN);
  size_t pitch = 0;
  hella::alloc_gpu_pitch<half>(&p.batch, &pitch, (size_t)w, NBATCH * NCHAN);
  hella::alloc_gpu_pitch<half>(&p.mask, &pitch, (size_t)w, NBATCH * NCHAN);
  p.batch_stride = (int)(pitch / sizeof(half));
  hella::alloc_gpu<half>(&p.d_smooth, (size_t)p.batch_stride * NBATCH * NCHAN);
  hella::alloc_gpu<float>(&p.d_ts, (size_t)w * NBATCH);
  hella::alloc_gpu<float>(&p.d_flagSpec, NCHAN * NBATCH);
  std::memset(p.d_flagSpec, 0, sizeof(float) * NCHAN * NBATCH);
  hella::alloc_cpu<float>(&p.h_flagSpec, NCHAN * NBATCH);
  hella::fast_flagger(&p);
  std::memcpy(out, p.d_data, (size_t)w * NCHAN);
  std::memcpy(ts, p.d_ts, sizeof(float) * w);
  std::memcpy(flagspec, p.h_flagSpec, sizeof(float) * NCHAN);
  return 0;
}

/* calculate_stddev<float / half> (normalization.cu:125-162). */
float ref_stddev_f32(const float *x, int width, int height, int stride, float *mean) {
  hella::pinfo_t p{};
  std::vector<float> buf(x, x + (size_t)height * stride);
  return hella::calculate_stddev<float>(&p, buf.data(), width, height, stride, mean);
}

float ref_stddev_f16(const uint16_t *x, int width, int height, int stride, float *mean) {
  hella::pinfo_t p{};
  std::vector<half> buf((size_t)height * stride);
  std::memcpy(buf.data(), x, buf.size() * sizeof(half));
  return hella::calculate_stddev<half>(&p, buf.data(), width, height, stride, mean);
}

/* median_filter (median_filter.cpp:38-83). */
float ref_median_filter(const float *in, float *out, int size, int window) {
  std::vector<float> buf(in, in + size);
  return hella::median_filter(buf.data(), out, size, window);
}

/* smooth(p, 1) (smooth.cpp:21-127) on a dedispersed plane [ndms][ntime_dd];
 * boxes out packed [nbox][ndms-2][ntime_out]; the smoothing kernels the
 * reference built (3 x (2sm+1) per width) are returned in order. */
int ref_smooth(const float *dd, int ndms, int ntime_dd, int ntime_out, int wmin, int wmax, float *boxes,
               float *taps, int taps_cap) {
  hella::pinfo_t p{};
  p.ndms = ndms;
  p.ntime_dd = ntime_dd;
  p.ntime_out = ntime_out;
  p.minWidth = wmin;
  p.maxWidth = wmax;
  p.nboxcar = 0;
  for (int i = wmin; i < wmax; i *= 2) p.nboxcar++;
  size_t step = 0;
  hella::alloc_gpu_pitch<float>(&p.d_dedisp, &step, (size_t)ntime_dd, ndms);
  p.d_dedisp_step = (int)step;
  for (int r = 0; r < ndms; ++r)
    std::memcpy(reinterpret_cast<char *>(p.d_dedisp) + r * step, dd + (size_t)r * ntime_dd, sizeof(float) * ntime_dd);
  hella::alloc_gpu_pitch<float>(&p.imbox, &step, (size_t)ntime_dd, ndms);
  p.imbox_step = (int)step;
  hella::alloc_gpu_pitch<float>(&p.boxes, &step, (size_t)ntime_out, (size_t)(ndms - 2) * p.nboxcar);
  p.boxes_step = (int)step;
  g_taps_seen.clear();
  hella::smooth(&p, 1);
  for (int b = 0; b < p.nboxcar; ++b)
    for (int r = 0; r < ndms - 2; ++r)
      std::memcpy(boxes + ((size_t)b * (ndms - 2) + r) * ntime_out,
                  reinterpret_cast<char *>(p.boxes) + ((size_t)b * (ndms - 2) + r) * p.boxes_step,
                  sizeof(float) * ntime_out);
  const int n = (int)g_taps_seen.size() < taps_cap ? (int)g_taps_seen.size() : taps_cap;
  std::memcpy(taps, g_taps_seen.data(), sizeof(float) * n);
  return p.nboxcar;
}

/* find_peaks (peaks.cu:31-117) on normalised boxes [nbox][ndms-2][ntime_out]:
 * candidates in the reference's order (snr, width, dm_idx, samp). */
int ref_find_peaks(const float *boxes, int nbox, int ndms, int ntime_out, float snr, int beam, float *o_snr,
                   int *o_width, int *o_dm, int *o_samp) {
  hella::pinfo_t p{};
  p.ndms = ndms;
  p.ntime_out = ntime_out;
  p.nboxcar = nbox;
  p.snr = snr;
  size_t step = 0;
  hella::alloc_gpu_pitch<float>(&p.boxes, &step, (size_t)ntime_out, (size_t)(ndms - 2) * nbox);
  p.boxes_step = (int)step;
  for (size_t r = 0; r < (size_t)(ndms - 2) * nbox; ++r)
    std::memcpy(reinterpret_cast<char *>(p.boxes) + r * step, boxes + r * ntime_out, sizeof(float) * ntime_out);
  p.dmt.resize((size_t)(ndms - 2) * ntime_out);
  p.output_indices.resize((size_t)(ndms - 2) * ntime_out);
  p.output_values.resize((size_t)(ndms - 2) * ntime_out);
  hella::alloc_cpu<int>(&p.h_idxs, (size_t)(ndms - 2) * ntime_out);
  hella::alloc_cpu<float>(&p.peaks, MAX_GIANTS);
  hella::alloc_cpu<int>(&p.out_beam, MAX_GIANTS);
  hella::alloc_cpu<int>(&p.out_samp, MAX_GIANTS);
  hella::alloc_cpu<int>(&p.out_width, MAX_GIANTS);
  hella::alloc_cpu<int>(&p.out_dm_idx, MAX_GIANTS);
  hella::alloc_cpu<float>(&p.out_peaks, MAX_GIANTS);
  hella::clear_peaks(&p);
  hella::find_peaks(&p, beam);
  for (int i = 0; i < p.out_npeaks; ++i) {
    o_snr[i] = p.out_peaks[i];
    o_width[i] = p.out_width[i];
    o_dm[i] = p.out_dm_idx[i];
    o_samp[i] = p.out_samp[i];
  }
  return p.out_npeaks;
}

}  // extern "C"
