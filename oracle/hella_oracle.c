/*
 * hella_oracle.c -- CPU restatement of casm-hella's per-gulp FRB search.
 *
 * TEST INFRASTRUCTURE ONLY (compared against, never the product): see
 * hella_oracle.h for the contract, the arithmetic conventions and what is
 * pinned.  Build: oracle/Makefile (gcc -O3 -fopenmp -ffp-contract=off).
 */
#include "hella_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;
void ho_set_threads(int n) { g_threads = n; }
static int nthreads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ fp16 */

uint16_t ho_f2h(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
  uint32_t ax = x & 0x7fffffffu;
  if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7fffu); /* NaN */
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* >= 65520: inf */
  if (ax < 0x38800000u) {                                  /* < 2^-14 */
    float af;
    memcpy(&af, &ax, 4);
    float s = af * 16777216.0f; /* |f| / 2^-24, exact */
    uint32_t m = (uint32_t)s;
    float frac = s - (float)m;
    if (frac > 0.5f || (frac == 0.5f && (m & 1u))) m++;
    return (uint16_t)(sign | m);
  }
  uint32_t h = (((ax >> 23) - 112u) << 10) | ((ax & 0x7fffffu) >> 13);
  uint32_t rem = ax & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}

float ho_h2f(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu, x;
  float f;
  if (e == 0) {
    f = (float)m * 5.9604644775390625e-8f; /* m * 2^-24 */
    memcpy(&x, &f, 4);
    x |= sign;
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112u) << 23) | (m << 13);
  }
  memcpy(&f, &x, 4);
  return f;
}

uint16_t ho_hadd(uint16_t a, uint16_t b) { return ho_f2h(ho_h2f(a) + ho_h2f(b)); }
uint16_t ho_hmul(uint16_t a, uint16_t b) { return ho_f2h(ho_h2f(a) * ho_h2f(b)); }
uint16_t ho_hdiv(uint16_t a, uint16_t b) { return ho_f2h(ho_h2f(a) / ho_h2f(b)); }

#define H_ONE ((uint16_t)0x3c00u)
#define H_ZERO ((uint16_t)0x0000u)

/* ------------------------------------------------------ dedisp plan math */

/*
 * DM trial spacing from a smearing tolerance (Cordes & McLaughlin 2003,
 * the rule used by brute-force dedispersion codes, Barsdell et al. 2012).
 * The effective width of a pulse of intrinsic width ti observed at trial DM
 * D with samples of length ts is W(D)^2 = ts^2 + ti^2 + (a D)^2, where
 * a = 8.3 us * |df|_MHz / f_GHz^3 is the in-channel smearing per unit DM at
 * the band centre.  A DM error e smears the pulse across the band by b*e
 * with b = a*nchan/4.  The next trial D' is the one for which the smearing
 * of a pulse at D' seen by trial D stays within tol*W(D):
 *     ts^2 + ti^2 + a^2 D'^2 + b^2 (D'-D)^2 = tol^2 (ts^2 + ti^2 + a^2 D^2).
 * Its larger root is
 *     D' = (b^2 D + sqrt(-a^2 b^2 D^2 + (a^2+b^2)(c + tol^2 a^2 D^2)))
 *          / (a^2 + b^2),     c = (ts^2 + ti^2)(tol^2 - 1).
 * Trials start at dm_start and stop at the first one >= dm_end (call site
 * casm_hella_refactored.cu:207, DM_TOL default 1.3 at :68).
 */
int ho_generate_dm_list(float *out, int max_out, double dm_start, double dm_end,
                        double ti_us, double tol, int nchan, double dt_s,
                        double f0_mhz, double df_mhz) {
  double ts = dt_s * 1e6;
  double adf = fabs(df_mhz);
  double f = (f0_mhz - (nchan * 0.5 - 0.5) * adf) * 1e-3;
  double tol2 = tol * tol;
  double a = 8.3 * adf / (f * f * f);
  double a2 = a * a;
  double b2 = a2 * (double)nchan * (double)nchan / 16.0;
  double c = (ts * ts + ti_us * ti_us) * (tol2 - 1.0);
  double dm = dm_start;
  int n = 0;
  if (max_out < 1) return -1;
  out[n++] = (float)dm;
  while (dm < dm_end) {
    double d2 = dm * dm;
    double k = c + tol2 * a2 * d2;
    dm = (b2 * dm + sqrt(-a2 * b2 * d2 + (a2 + b2) * k)) / (a2 + b2);
    if (n >= max_out) return -1;
    out[n++] = (float)dm;
  }
  return n;
}

/* Cold-plasma delay relative to channel 0: K_DM (1/f_c^2 - 1/f0^2) / dt. */
void ho_delay_table(float *table, int nchan, double dt_s, double f0_mhz,
                    double df_mhz) {
  double adf = fabs(df_mhz);
  for (int c = 0; c < nchan; ++c) {
    double fc = f0_mhz - c * adf;
    table[c] = (float)(HO_KDM / dt_s * (1.0 / (fc * fc) - 1.0 / (f0_mhz * f0_mhz)));
  }
}

/* Delay rounded to the nearest sample: (int)(DM * table + 0.5f) in fp32. */
void ho_dm_delays(int32_t *delays, const float *dms, int ndms,
                  const float *table, int nchan) {
  for (int d = 0; d < ndms; ++d)
    for (int c = 0; c < nchan; ++c) {
      float p = dms[d] * table[c];
      p = p + 0.5f;
      delays[(size_t)d * nchan + c] = (int32_t)p;
    }
}

/* ------------------------------------------------------------ dedisperse */

void ho_dedisperse(const uint8_t *in, int nsamps, size_t in_stride, int nchan,
                   const int32_t *delays, int ndms, const int32_t *killmask,
                   float *out, size_t out_stride, int nout) {
  /* Channel-major copy so each DM trial streams contiguous rows. */
  uint8_t *ft = (uint8_t *)malloc((size_t)nchan * nsamps);
  for (int t = 0; t < nsamps; ++t)
    for (int c = 0; c < nchan; ++c) ft[(size_t)c * nsamps + t] = in[(size_t)t * in_stride + c];
#pragma omp parallel num_threads(nthreads())
  {
    uint32_t *acc = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)nout);
#pragma omp for schedule(dynamic, 4)
    for (int d = 0; d < ndms; ++d) {
      memset(acc, 0, sizeof(uint32_t) * (size_t)nout);
      for (int c = 0; c < nchan; ++c) {
        if (killmask && !killmask[c]) continue;
        const uint8_t *row = ft + (size_t)c * nsamps + delays[(size_t)d * nchan + c];
        for (int t = 0; t < nout; ++t) acc[t] += row[t];
      }
      float *o = out + (size_t)d * out_stride;
      for (int t = 0; t < nout; ++t) o[t] = (float)acc[t];
    }
    free(acc);
  }
  free(ft);
}

/* ------------------------------------------------------------ statistics */

/* Lane 0 after __shfl_down_sync offsets 16,8,4,2,1 (normalization.cu:46-47,
 * flagger.cu:103-106).  Lanes whose source is out of range keep adding their
 * own value, as the shuffle returns it; lane 0 never reads such a lane. */
static float warp_tree(const float *v32) {
  float v[32];
  memcpy(v, v32, sizeof v);
  for (int off = 16; off > 0; off /= 2)
    for (int l = 0; l < 32; ++l) v[l] = v[l] + (l + off < 32 ? v[l + off] : v[l]);
  return v[0];
}

/* Thread 0 of a 256-thread row block: its warp's total, then the other
 * warps' totals in order (normalization.cu:51-68). */
static float block256_sum(const float *p) {
  float s = warp_tree(p);
  for (int w = 1; w < 8; ++w) s += warp_tree(p + 32 * w);
  return s;
}

#define STDDEV_IMPL(NAME, T, GET)                                              \
  float NAME(const T *data, int width, int height, size_t stride,              \
             float *mean_out) {                                                \
    int nw = 256 * (width / 256);                                              \
    float *rows = (float *)malloc(sizeof(float) * (size_t)height);             \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads())")       \
    for (int r = 0; r < height; ++r) {                                         \
      float p[256] = {0};                                                      \
      const T *row = data + (size_t)r * stride;                                \
      for (int k = 0; k < nw; k += 256)                                        \
        for (int j = 0; j < 256; ++j) p[j] += GET(row[k + j]);                 \
      rows[r] = block256_sum(p) / (float)nw;                                   \
    }                                                                          \
    float mean = 0.f;                                                          \
    for (int r = 0; r < height; ++r) mean += rows[r];                          \
    mean /= (float)height;                                                     \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads())")       \
    for (int r = 0; r < height; ++r) {                                         \
      float p[256] = {0};                                                      \
      const T *row = data + (size_t)r * stride;                                \
      for (int k = 0; k < nw; k += 256)                                        \
        for (int j = 0; j < 256; ++j) {                                        \
          float v = GET(row[k + j]) - mean;                                    \
          p[j] = fmaf(v, v, p[j]);                                             \
        }                                                                      \
      rows[r] = block256_sum(p) / (float)nw;                                   \
    }                                                                          \
    float var = 0.f;                                                           \
    for (int r = 0; r < height; ++r) var += rows[r];                           \
    var /= (float)height;                                                      \
    free(rows);                                                                \
    if (mean_out) *mean_out = mean;                                            \
    return sqrtf(var);                                                         \
  }

#define GET_F32(x) (x)
#define GET_F16(x) ho_h2f(x)
STDDEV_IMPL(ho_stddev_f32, float, GET_F32)
STDDEV_IMPL(ho_stddev_f16, uint16_t, GET_F16)

/* --------------------------------------------------------------- flagger
 * The batch is fp16 [nchan][w] with row stride w (a pitched allocation
 * whose pitch equals the row, true whenever 2w is a multiple of the pitch
 * alignment). */

/* calc_bandpass_new  flagger.cu:86-112: lane l sums columns l, l+32, ...
 * below 32*floor(w/32); warp tree; divided by w (not the count summed). */
static void calc_bandpass_new(const uint16_t *d, int nchan, int w, float *bp) {
  int np = w / 32;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int c = 0; c < nchan; ++c) {
    float lane[32];
    const uint16_t *row = d + (size_t)c * w;
    for (int l = 0; l < 32; ++l) {
      float s = 0.f;
      for (int i = 0; i < np; ++i) s += ho_h2f(row[l + 32 * i]);
      lane[l] = s;
    }
    bp[c] = warp_tree(lane) / (float)w;
  }
}

/* median_filter  median_filter.cpp:38-83 (bubble sort, odd window, edges
 * copied from the nearest filtered value); returns the mean of the output. */
static float median_filter(const float *in, float *out, int size, int win) {
  int h = win / 2;
  float window[64];
  for (int i = h; i < size - h; ++i) {
    int n = 0;
    for (int j = i - h; j <= i + h; ++j) window[n++] = (j >= 0 && j < size) ? in[j] : in[i];
    for (int a = 0; a < win - 1; ++a)
      for (int b = 0; b < win - a - 1; ++b)
        if (window[b] > window[b + 1]) {
          float t = window[b];
          window[b] = window[b + 1];
          window[b + 1] = t;
        }
    out[i] = (win % 2) ? window[win / 2] : (window[(win - 1) / 2] + window[win / 2]) / 2.0f;
  }
  for (int i = 0; i < h; ++i) out[i] = out[h];
  for (int i = size - h; i < size; ++i) out[i] = out[size - h - 1];
  float mn = 0.f;
  for (int i = 0; i < size; ++i) mn += out[i];
  return mn / (float)(1. * size);
}

float ho_median_filter(const float *in, float *out, int size, int window) {
  return median_filter(in, out, size, window);
}

/* bandpass_correct  flagger.cu:244-269 (+ med_filter_bandpass
 * median_filter.cpp:85-107 with a window of NMEDFILT, definitions.h:39: 1,
 * the identity, in the reference's build) and divide_by_bp
 * flagger.cu:180-194. */
static void bandpass_correct(uint16_t *d, int nchan, int w, float *bp_out, int nmedfilt) {
  float *bp = (float *)malloc(sizeof(float) * (size_t)nchan);
  float *mbp = (float *)malloc(sizeof(float) * (size_t)nchan);
  calc_bandpass_new(d, nchan, w, bp);
  median_filter(bp, mbp, nchan, nmedfilt > 1 ? nmedfilt : 1);
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int c = 0; c < nchan; ++c) {
    uint16_t *row = d + (size_t)c * w;
    if (mbp[c] > 0) {
      uint16_t hb = ho_f2h(mbp[c]);
      for (int t = 0; t < w; ++t) row[t] = ho_hdiv(row[t], hb);
    } else {
      for (int t = 0; t < w; ++t) row[t] = H_ZERO;
    }
  }
  if (bp_out) memcpy(bp_out, mbp, sizeof(float) * (size_t)nchan);
  free(bp);
  free(mbp);
}

/* normalize_data  flagger.cu:198-214: x = (x + half(-mean)) * half(1/std). */
static void normalize_data(uint16_t *d, int nchan, int w, float *mean_o, float *std_o) {
  float mean = 0.f;
  float sd = ho_stddev_f16(d, w, nchan, (size_t)w, &mean);
  uint16_t a = ho_f2h(-mean);
  uint16_t m = ho_f2h(1.f / sd);
  size_t n = (size_t)nchan * w;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (size_t i = 0; i < n; ++i) d[i] = ho_hmul(ho_hadd(d[i], a), m);
  if (mean_o) *mean_o = mean;
  if (std_o) *std_o = sd;
}

/* ts_correct  timeseries.cu:19-74: fp16 running sum over channels (in
 * channel order) / nchan, then every channel divided by half(ts[t]). */
static void ts_correct(uint16_t *d, int nchan, int w, float *ts_out) {
  float *ts = (float *)malloc(sizeof(float) * (size_t)w);
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int t = 0; t < w; ++t) {
    uint16_t s = H_ZERO;
    for (int c = 0; c < nchan; ++c) s = ho_hadd(s, d[(size_t)c * w + t]);
    ts[t] = ho_h2f(s) / (float)nchan;
  }
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int c = 0; c < nchan; ++c)
    for (int t = 0; t < w; ++t) d[(size_t)c * w + t] = ho_hdiv(d[(size_t)c * w + t], ho_f2h(ts[t]));
  if (ts_out) memcpy(ts_out, ts, sizeof(float) * (size_t)w);
  free(ts);
}

/* npp_convolve_handler  convolution.cu:20-55: uniform xw (time) x yw
 * (channel) box of taps `k`, anchor (xw/2, yw/2), replicate border, fp32
 * accumulation of fp16 input, fp16 output.  Tap (j, i) multiplies input
 * (c + ay - j, t + ax - i), the placement nppiFilterBorder uses (an impulse
 * response measured on a GB300); the summation order (j outer, i inner,
 * one fmaf per tap) is this project's definition. */
static void box_filter(const uint16_t *in, uint16_t *out, int nchan, int w,
                       int xw, int yw, float k) {
  int ax = xw / 2, ay = yw / 2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int c = 0; c < nchan; ++c)
    for (int t = 0; t < w; ++t) {
      float acc = 0.f;
      for (int j = 0; j < yw; ++j) {
        int cc = c + ay - j;
        cc = cc < 0 ? 0 : (cc >= nchan ? nchan - 1 : cc);
        for (int i = 0; i < xw; ++i) {
          int tt = t + ax - i;
          tt = tt < 0 ? 0 : (tt >= w ? w - 1 : tt);
          acc = fmaf(k, ho_h2f(in[(size_t)cc * w + tt]), acc);
        }
      }
      out[(size_t)c * w + t] = ho_f2h(acc);
    }
}

void ho_box_filter(const uint16_t *in, uint16_t *out, int nchan, int w, int xw,
                   int yw, float k) {
  box_filter(in, out, nchan, w, xw, yw, k);
}

/* calc_bandpass  flagger.cu:50-81: 256 threads per channel, thread t sums
 * its contiguous chunk of floor(w/256) samples in fp16, divides by
 * half(256*floor(w/256)), then an fp16 shared-memory tree. */
static void calc_bandpass_f16(const uint16_t *d, int nchan, int w, float *bp) {
  int np = w / 256;
  uint16_t fac = ho_f2h((float)(256. * np));
  for (int c = 0; c < nchan; ++c) {
    uint16_t ps[256];
    for (int t = 0; t < 256; ++t) {
      uint16_t s = H_ZERO;
      const uint16_t *p = d + (size_t)c * w + (size_t)t * np;
      for (int i = 0; i < np; ++i) s = ho_hadd(s, p[i]);
      ps[t] = ho_hdiv(s, fac);
    }
    for (int s = 128; s >= 1; s /= 2)
      for (int t = 0; t < s; ++t) ps[t] = ho_hadd(ps[t], ps[t + s]);
    bp[c] = ho_h2f(ps[0]);
  }
}

/* apply_scrunch  flagger.cu:271-343. */
static void apply_scrunch(uint16_t *d, uint16_t *mask, uint16_t *smooth,
                          int nchan, int w, int tscr, int fscr, float thresh,
                          int flag, int ts, const ho_flag_params *fp,
                          float *flagspec, float *bp_out, float *ts_out,
                          float *mean_o, float *std_o) {
  bandpass_correct(d, nchan, w, bp_out, fp->bp_median);
  if (ts == 1) ts_correct(d, nchan, w, ts_out);
  normalize_data(d, nchan, w, mean_o, std_o);
  if (flag == 1) {
    size_t n = (size_t)nchan * w;
    float k = (float)(1. / tscr / fscr);
    box_filter(d, smooth, nchan, w, tscr, fscr, k);
    memset(mask, 0, n * sizeof(uint16_t));
    float thr = (float)(thresh / sqrt(1. * tscr * fscr));
    uint16_t hp = ho_f2h(thr), hn = ho_f2h((float)(-1. * thr));
    for (size_t i = 0; i < n; ++i) {
      if (ho_h2f(smooth[i]) > ho_h2f(hp)) mask[i] = H_ONE;
      if (ho_h2f(smooth[i]) < ho_h2f(hn)) mask[i] = H_ONE;
    }
    box_filter(mask, smooth, nchan, w, tscr, fscr, k);
    for (int c = 0; c < nchan; ++c)
      for (int t = 0; t < w; ++t) {
        size_t i = (size_t)c * w + t;
        if (ho_h2f(smooth[i]) > 0.f) d[i] = H_ZERO;
        if (c >= fp->flag1 && c < fp->flag2) d[i] = H_ZERO;
      }
    for (size_t i = 0; i < n; ++i) d[i] = ho_hadd(d[i], H_ONE);
    if (flagspec) {
      float *dm = (float *)malloc(sizeof(float) * (size_t)nchan);
      calc_bandpass_f16(smooth, nchan, w, dm);
      for (int c = 0; c < nchan; ++c) flagspec[c] += dm[c];
      free(dm);
    }
  }
}

/* transpose_output  transpose.cu:48-76: u8 = trunc(clamp(255/14 (x+4))). */
static uint8_t requant(uint16_t h) {
  float v = ho_h2f(h);
  const float scf = 255.f / 14.f;
  v = scf * (v + 4.f);
  if (v < 0.) v = 0;
  if (v > 255.f) v = 255.f;
  if (v != v) return 0; /* NaN converts to 0 (cvt.rzi semantics) */
  return (uint8_t)v;
}

/* fast_flagger (flagger.cu:345-411) from the fp16 channel-major copy d of
 * one beam's gulp, which it consumes. */
static void flag_plane(uint16_t *d, int w, int nchan, const ho_flag_params *fp, uint8_t *out,
                       float *ts_out, float *flagspec, ho_flag_trace *tr);

void ho_flag_beam(const uint8_t *gulp, int w, int nchan,
                  const ho_flag_params *fp, uint8_t *out, float *ts_out,
                  float *flagspec, ho_flag_trace *tr) {
  size_t n = (size_t)nchan * w;
  uint16_t *d = (uint16_t *)malloc(n * sizeof(uint16_t));
  /* transpose_input  transpose.cu:23-42 (u8 -> fp16, exact) */
  for (int t = 0; t < w; ++t)
    for (int c = 0; c < nchan; ++c) d[(size_t)c * w + t] = ho_f2h((float)gulp[(size_t)t * nchan + c]);
  flag_plane(d, w, nchan, fp, out, ts_out, flagspec, tr);
  free(d);
}

/* The DADA input path (transpose_input_handler, transpose.cu:87-90): the
 * gulp arrives as fp16 in channel-major (FT) order and is flagged as is. */
void ho_flag_beam_f16(const uint16_t *ft, int w, int nchan, const ho_flag_params *fp,
                      uint8_t *out, float *ts_out, float *flagspec, ho_flag_trace *tr) {
  size_t n = (size_t)nchan * w;
  uint16_t *d = (uint16_t *)malloc(n * sizeof(uint16_t));
  memcpy(d, ft, n * sizeof(uint16_t));
  flag_plane(d, w, nchan, fp, out, ts_out, flagspec, tr);
  free(d);
}

static void flag_plane(uint16_t *d, int w, int nchan, const ho_flag_params *fp, uint8_t *out,
                       float *ts_out, float *flagspec, ho_flag_trace *tr) {
  size_t n = (size_t)nchan * w;
  uint16_t *mask = (uint16_t *)malloc(n * sizeof(uint16_t));
  uint16_t *sm = (uint16_t *)malloc(n * sizeof(uint16_t));
  float *bp = (float *)malloc(sizeof(float) * (size_t)nchan);
  float m1, s1, m2, s2;
  /* bandpass_flag  flagger.cu:216-242 */
  bandpass_correct(d, nchan, w, tr ? tr->bp1 : NULL, fp->bp_median);
  normalize_data(d, nchan, w, &m1, &s1);
  calc_bandpass_new(d, nchan, w, bp);
  for (int c = 0; c < nchan; ++c) {
    uint16_t *row = d + (size_t)c * w;
    if (bp[c] < fp->spec_min || bp[c] > fp->spec_max) {
      for (int t = 0; t < w; ++t) row[t] = H_ONE;
    } else {
      for (int t = 0; t < w; ++t) row[t] = ho_hadd(row[t], H_ONE);
    }
  }
  if (tr) {
    memcpy(tr->bp2, bp, sizeof(float) * (size_t)nchan);
    tr->mean1 = m1;
    tr->std1 = s1;
  }
  /* user scrunches, then the fixed final one (flagger.cu:365-401) */
  for (int i = 0; i < fp->nscrunch; ++i) {
    const ho_scrunch *s = &fp->scrunches[i];
    apply_scrunch(d, mask, sm, nchan, w, s->tscrunch, s->fscrunch, s->thresh, 1, 0,
                  fp, flagspec, NULL, NULL, NULL, NULL);
  }
  apply_scrunch(d, mask, sm, nchan, w, 8, 8, 100.f, 0, 1, fp, flagspec,
                tr ? tr->bp3 : NULL, ts_out, &m2, &s2);
  if (tr) {
    tr->mean2 = m2;
    tr->std2 = s2;
  }
  for (int t = 0; t < w; ++t)
    for (int c = 0; c < nchan; ++c) out[(size_t)t * nchan + c] = requant(d[(size_t)c * w + t]);
  free(mask);
  free(sm);
  free(bp);
}

/* ------------------------------------------------------------- smoothing */

int ho_smooth_taps(int sm, float *k) {
  const float wt[3] = {0.3f, 1.f, 0.3f};
  int n = 2 * sm + 1;
  float filtSum = 0.f;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < n; ++j) {
      double u = (j - sm) / (sm / 2.355);
      float v = (float)(1. - 0.5 * u * u + 0.25 * u * u * 0.25 * u * u -
                        0.083 * u * u * 0.083 * u * u * 0.083 * u * u);
      float kv = wt[i] * v * v;
      k[i * n + j] = kv;
      filtSum += kv;
    }
  for (int i = 0; i < 3 * n; ++i) k[i] /= filtSum;
  return n;
}

void ho_smooth_plane(const float *dd, int ndms, int ntime_dd, size_t dd_stride,
                     int sm, int wmax, int shift, float *out, int ntime_out,
                     size_t out_stride) {
  float *k3 = (float *)malloc(sizeof(float) * 3 * (2 * sm + 1));
  int n = ho_smooth_taps(sm, k3);
  const float *km = k3 + n; /* middle (DM weight 1) row */
#pragma omp parallel num_threads(nthreads())
  {
    float *y = (float *)malloc(sizeof(float) * (size_t)ntime_dd);
#pragma omp for schedule(static)
    for (int r = 0; r < ndms - 2; ++r) {
      const float *a = dd + (size_t)r * dd_stride;
      const float *b = a + dd_stride;
      const float *c = b + dd_stride;
      for (int x = 0; x < ntime_dd; ++x) y[x] = fmaf(0.3f, a[x] + c[x], b[x]);
      float *o = out + (size_t)r * out_stride;
      for (int j = 0; j < ntime_out; ++j) {
        int x0 = j + wmax / 2 - shift;
        float acc = 0.f;
        for (int q = 0; q < n; ++q) {
          int x = x0 + q;
          x = x < 0 ? 0 : (x >= ntime_dd ? ntime_dd - 1 : x);
          acc = fmaf(km[q], y[x], acc);
        }
        o[j] = acc;
      }
    }
    free(y);
  }
  free(k3);
}

void ho_smooth_plane_direct(const float *dd, int ndms, int ntime_dd,
                            size_t dd_stride, int sm, int wmax, int shift,
                            float *out, int ntime_out, size_t out_stride) {
  float *k3 = (float *)malloc(sizeof(float) * 3 * (2 * sm + 1));
  int n = ho_smooth_taps(sm, k3);
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int r = 0; r < ndms - 2; ++r) {
    float *o = out + (size_t)r * out_stride;
    for (int j = 0; j < ntime_out; ++j) {
      /* output column x = j + wmax/2 of dd row r+1 */
      int x = j + wmax / 2;
      float acc = 0.f;
      for (int kr = 0; kr < 3; ++kr) {
        const float *row = dd + (size_t)(r + 2 - kr) * dd_stride;
        for (int i = 0; i < n; ++i) {
          int xx = x + (2 * sm - shift) - i; /* column i on input x - i (anchor 1) */
          xx = xx < 0 ? 0 : (xx >= ntime_dd ? ntime_dd - 1 : xx);
          acc = fmaf(k3[kr * n + i], row[xx], acc);
        }
      }
      o[j] = acc;
    }
  }
  free(k3);
}

int ho_smooth_normalise_arith(const float *dd, int ndms, int ntime_dd,
                              size_t dd_stride, int wmin, int wmax, int anchor,
                              int ntime_out, float *boxes, float *mean,
                              float *std, int direct) {
  int nb = 0;
  size_t plane = (size_t)(ndms - 2) * ntime_out;
  for (int sm = wmin; sm < wmax; sm *= 2, ++nb)
    (direct ? ho_smooth_plane_direct : ho_smooth_plane)(
        dd, ndms, ntime_dd, dd_stride, sm, wmax, anchor ? 2 * sm : 0,
        boxes + nb * plane, ntime_out, (size_t)ntime_out);
  for (int b = 0; b < nb; ++b) {
    float *x = boxes + b * plane;
    float mu = 0.f;
    float sd = ho_stddev_f32(x, ntime_out, ndms - 2, (size_t)ntime_out, &mu);
    if (mean) mean[b] = mu;
    if (std) std[b] = sd;
    if (sd > 0) { /* smooth.cpp:105-123: AddC(-mean) then MulC(1/std) */
      float nm = -1.0f * mu, r = 1.0f / sd;
#pragma omp parallel for schedule(static) num_threads(nthreads())
      for (size_t i = 0; i < plane; ++i) {
        float v = x[i] + nm;
        x[i] = v * r;
      }
    }
  }
  return nb;
}

int ho_smooth_normalise(const float *dd, int ndms, int ntime_dd,
                        size_t dd_stride, int wmin, int wmax, int anchor,
                        int ntime_out, float *boxes, float *mean, float *std) {
  return ho_smooth_normalise_arith(dd, ndms, ntime_dd, dd_stride, wmin, wmax,
                                   anchor, ntime_out, boxes, mean, std, 0);
}

/* ----------------------------------------------------------------- peaks */

int ho_find_peaks(const float *boxes, int nbox, int ndms, int ntime_out,
                  float snr, int beam, int cap, ho_cand *out, float *sigma0) {
  return ho_find_peaks_gate(boxes, nbox, ndms, ntime_out, snr, beam, cap, out, sigma0, 1);
}

int ho_find_peaks_gate(const float *boxes, int nbox, int ndms, int ntime_out,
                       float snr, int beam, int cap, ho_cand *out, float *sigma0,
                       int gate) {
  int h = ndms - 2;
  size_t plane = (size_t)h * ntime_out;
  float mean = 0.f;
  float s0 = ho_stddev_f32(boxes, ntime_out, h, (size_t)ntime_out, &mean);
  if (sigma0) *sigma0 = s0;
  if (gate && !(s0 < 5 && s0 > 0.1)) return 0; /* definitions.h:66,71-72, peaks.cu:60 */
  float thr = snr * s0;
  int n = 0;
  for (int b = 0; b < nbox && n < cap; ++b) {
    const float *x = boxes + b * plane;
    for (size_t i = 0; i < plane && n < cap; ++i)
      if (x[i] > thr) {
        out[n].beam = beam;
        out[n].width = b;
        out[n].dm_idx = (int32_t)(i / ntime_out) + 1;
        out[n].samp = (int32_t)(i % ntime_out);
        out[n].snr = x[i];
        ++n;
      }
  }
  return n;
}

/* ------------------------------------------------------------- pipeline */

struct ho_pipeline {
  ho_params p;
  int ntime, ndms, max_delay, ntime_dd, nbox, min_gulp, gulp_idx;
  float *dms, *table;
  int32_t *delays;
  int32_t *killmask; /* [nbeam][nchan] or NULL (every channel summed) */
  uint8_t *ring;
  float *flagspec;
};

ho_pipeline *ho_pipeline_create(const ho_params *p) {
  ho_pipeline *pl = (ho_pipeline *)calloc(1, sizeof(ho_pipeline));
  pl->p = *p;
  /* the plan API takes fp32 band parameters (dedisp_create_plan) */
  const double dt = (float)p->plan_dt, f0 = (float)p->f0_mhz, df = (float)p->df_mhz;
  float *tmp = (float *)malloc(sizeof(float) * 1000000);
  int nd = ho_generate_dm_list(tmp, 1000000, p->dm_min, p->dm_max, p->ti_us, p->dm_tol,
                               p->nchan, dt, f0, df);
  if (nd < 3) {
    free(tmp);
    free(pl);
    return NULL;
  }
  pl->ndms = nd;
  pl->dms = (float *)malloc(sizeof(float) * nd);
  memcpy(pl->dms, tmp, sizeof(float) * nd);
  free(tmp);
  pl->table = (float *)malloc(sizeof(float) * p->nchan);
  ho_delay_table(pl->table, p->nchan, dt, f0, df);
  pl->delays = (int32_t *)malloc(sizeof(int32_t) * (size_t)nd * p->nchan);
  ho_dm_delays(pl->delays, pl->dms, nd, pl->table, p->nchan);
  pl->max_delay = pl->delays[(size_t)(nd - 1) * p->nchan + p->nchan - 1];
  /* casm_hella_refactored.cu:217-222 */
  pl->ntime = 32 * ((p->gulp + pl->max_delay + p->wmax) / 32 + 1);
  pl->ntime_dd = p->gulp + p->wmax;
  pl->nbox = 0;
  for (int sm = p->wmin; sm < p->wmax; sm *= 2) pl->nbox++;
  pl->min_gulp = pl->ntime / p->gulp; /* :632 */
  pl->ring = (uint8_t *)calloc((size_t)p->nbeam * pl->ntime * p->nchan, 1);
  pl->flagspec = (float *)calloc((size_t)p->nchan, sizeof(float));
  return pl;
}

void ho_pipeline_destroy(ho_pipeline *pl) {
  if (!pl) return;
  free(pl->dms);
  free(pl->table);
  free(pl->delays);
  free(pl->killmask);
  free(pl->ring);
  free(pl->flagspec);
  free(pl);
}

int ho_pipeline_info(const ho_pipeline *pl, int *ntime, int *ndms,
                     int *max_delay, int *ntime_dd, int *nbox, int *min_gulp) {
  if (ntime) *ntime = pl->ntime;
  if (ndms) *ndms = pl->ndms;
  if (max_delay) *max_delay = pl->max_delay;
  if (ntime_dd) *ntime_dd = pl->ntime_dd;
  if (nbox) *nbox = pl->nbox;
  if (min_gulp) *min_gulp = pl->min_gulp;
  return 0;
}

const float *ho_pipeline_dms(const ho_pipeline *pl) { return pl->dms; }
const int32_t *ho_pipeline_delays(const ho_pipeline *pl) { return pl->delays; }
const uint8_t *ho_pipeline_ring(const ho_pipeline *pl, int beam) {
  return pl->ring + (size_t)beam * pl->ntime * pl->p.nchan;
}
const float *ho_pipeline_flagspec(const ho_pipeline *pl) { return pl->flagspec; }

/* A dedisp plan's killmask for one beam (the reference holds one plan, so one
 * killmask, per process: casm_hella_refactored.cu:204-212). */
int ho_pipeline_set_killmask(ho_pipeline *pl, int beam, const int32_t *killmask) {
  const int nchan = pl->p.nchan;
  if (beam < 0 || beam >= pl->p.nbeam) return -1;
  if (!pl->killmask) {
    pl->killmask = (int32_t *)malloc(sizeof(int32_t) * (size_t)pl->p.nbeam * nchan);
    for (size_t i = 0; i < (size_t)pl->p.nbeam * nchan; ++i) pl->killmask[i] = 1;
  }
  for (int c = 0; c < nchan; ++c) pl->killmask[(size_t)beam * nchan + c] = killmask ? killmask[c] : 1;
  return 0;
}

int ho_search_window(const ho_pipeline *pl, const uint8_t *window, int beam,
                     int cap, ho_cand *cands, float *dd_out, float *boxes_out,
                     float *mean_out, float *std_out, float *sigma0) {
  const ho_params *p = &pl->p;
  size_t ddn = (size_t)pl->ndms * pl->ntime_dd;
  size_t bxn = (size_t)pl->nbox * (pl->ndms - 2) * p->gulp;
  float *dd = dd_out ? dd_out : (float *)malloc(sizeof(float) * ddn);
  float *bx = boxes_out ? boxes_out : (float *)malloc(sizeof(float) * bxn);
  /* dedisperse.cpp:17-48 (ntime_dedisp outputs, first ntime_dd kept) */
  ho_dedisperse(window, pl->ntime, (size_t)p->nchan, p->nchan, pl->delays, pl->ndms,
                pl->killmask ? pl->killmask + (size_t)beam * p->nchan : NULL, dd,
                (size_t)pl->ntime_dd, pl->ntime_dd);
  ho_smooth_normalise(dd, pl->ndms, pl->ntime_dd, (size_t)pl->ntime_dd, p->wmin, p->wmax,
                      p->smooth_anchor, p->gulp, bx, mean_out, std_out);
  int n = ho_find_peaks_gate(bx, pl->nbox, pl->ndms, p->gulp, p->snr, beam, cap, cands, sigma0,
                             !p->always_find_peaks);
  if (!dd_out) free(dd);
  if (!boxes_out) free(bx);
  return n;
}

static int pipeline_step(ho_pipeline *pl, const void *gulp, int f16, ho_cand *cands, int max_cands,
                         int *searched);

int ho_pipeline_gulp(ho_pipeline *pl, const uint8_t *gulp, ho_cand *cands,
                     int max_cands, int *searched) {
  return pipeline_step(pl, gulp, 0, cands, max_cands, searched);
}

/* The gulp loop fed fp16 FT gulps [nbeam][nchan][gulp] (DADA input). */
int ho_pipeline_gulp_f16(ho_pipeline *pl, const uint16_t *gulp, ho_cand *cands,
                         int max_cands, int *searched) {
  return pipeline_step(pl, gulp, 1, cands, max_cands, searched);
}

static int pipeline_step(ho_pipeline *pl, const void *gulp, int f16, ho_cand *cands, int max_cands,
                         int *searched) {
  const ho_params *p = &pl->p;
  size_t beam_ring = (size_t)pl->ntime * p->nchan;
  size_t beam_gulp = (size_t)p->gulp * p->nchan;
  int nout = 0;
  for (int b = 0; b < p->nbeam; ++b) {
    uint8_t *dst = pl->ring + b * beam_ring + (size_t)(pl->ntime - p->gulp) * p->nchan;
    if (f16)
      ho_flag_beam_f16((const uint16_t *)gulp + b * beam_gulp, p->gulp, p->nchan, &p->flag, dst, NULL,
                       pl->flagspec, NULL);
    else
      ho_flag_beam((const uint8_t *)gulp + b * beam_gulp, p->gulp, p->nchan, &p->flag, dst, NULL,
                   pl->flagspec, NULL);
  }
  int cap = p->max_giants < max_cands ? p->max_giants : max_cands;
  int do_search = pl->gulp_idx >= pl->min_gulp; /* :705 */
  if (do_search)
    for (int b = 0; b < p->nbeam && nout < cap; ++b) /* :723 */
      nout += ho_search_window(pl, pl->ring + b * beam_ring, b, cap - nout, cands + nout,
                               NULL, NULL, NULL, NULL, NULL);
  /* rewind :775-797 -- a left shift of every beam's ring by one gulp */
  for (int b = 0; b < p->nbeam; ++b)
    memmove(pl->ring + b * beam_ring, pl->ring + b * beam_ring + beam_gulp,
            beam_ring - beam_gulp);
  pl->gulp_idx++;
  if (searched) *searched = do_search;
  return nout;
}
