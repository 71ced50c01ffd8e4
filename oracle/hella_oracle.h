/*
 * hella_oracle.h -- CPU restatement of casm-hella's per-gulp FRB search.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU path is compared against this library:
 * only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * may load it.  The product (libhella_gb300.so) never links or calls it.
 *
 * Every function restates one piece of the reference (Coherent-All-Sky-
 * Monitor/casm-hella) and names the file:line it follows.  Arithmetic is
 * written out operation by operation so that fp16 and fp32 rounding follows
 * the reference kernels:
 *   - fp16 values are carried as IEEE binary16 bit patterns (uint16_t);
 *     every fp16 add/mul/div is computed in fp32 and rounded to fp16 once,
 *     which equals the correctly rounded fp16 result because 24 >= 2*11+2;
 *   - fp32 reductions follow the reference's thread/warp/host order;
 *   - multiply-adds that the reference's compiler fuses are written fmaf();
 *     nothing else is contracted (built with -ffp-contract=off).
 *
 * Pinning: the flagger, statistics, requantisation, smoothing taps and peak
 * decoding are pinned by golden fixtures generated from the reference's own
 * code (tests/golden).  The dedispersion plan (DM list, delay rounding,
 * output scaling) lives in the third-party dedisp library, which the
 * reference does not vendor and whose version it does not pin: that part is
 * restated from the published method and is "parity unpinned" against
 * dedisp itself (see the plan functions below).
 */
#ifndef HELLA_ORACLE_H
#define HELLA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- fp16 */
uint16_t ho_f2h(float f);          /* round-to-nearest-even float -> binary16 */
float ho_h2f(uint16_t h);          /* exact binary16 -> float */
uint16_t ho_hadd(uint16_t a, uint16_t b);
uint16_t ho_hmul(uint16_t a, uint16_t b);
uint16_t ho_hdiv(uint16_t a, uint16_t b);

/* ------------------------------------------------------- dedisp plan math
 * Restated from the published brute-force method (Barsdell et al. 2012) and
 * the Cordes & McLaughlin (2003) smearing model; dedisp's own source is not
 * part of the reference.  Call sites followed:
 * casm_hella_refactored.cu:205-210 (create plan, DM list, max delay).
 */
#define HO_KDM 4.148808e3 /* s MHz^2 / (pc cm^-3), make_noise_fil_with_frb.py:54 */

/* DM trials from dm_start until >= dm_end with smearing tolerance `tol` for
 * a pulse of width ti_us; returns the count (or -1 if > max_out). */
int ho_generate_dm_list(float *out, int max_out, double dm_start, double dm_end,
                        double ti_us, double tol, int nchan, double dt_s,
                        double f0_mhz, double df_mhz);
/* Per-channel delay in samples per unit DM; channel 0 is the highest
 * frequency f0, channel c is f0 - c*|df|. */
void ho_delay_table(float *table, int nchan, double dt_s, double f0_mhz,
                    double df_mhz);
/* delays[d*nchan + c] = (int)(dms[d]*table[c] + 0.5f) in fp32. */
void ho_dm_delays(int32_t *delays, const float *dms, int ndms,
                  const float *table, int nchan);

/* ------------------------------------------------------------ dedisperse
 * Brute-force direct dedispersion, dedisp_execute_adv as called at
 * dedisperse.cpp:17-48:  out[d][t] = sum over unkilled c of
 * in[t + delay(c,d)][c], t < nout, written as the exact integer in fp32.
 * in: u8 time-major, in_stride bytes per sample.  killmask may be NULL. */
void ho_dedisperse(const uint8_t *in, int nsamps, size_t in_stride, int nchan,
                   const int32_t *delays, int ndms, const int32_t *killmask,
                   float *out, size_t out_stride, int nout);

/* ------------------------------------------------------------ statistics
 * calculate_stddev<T>  normalization.cu:125-162 with computeRowMeans
 * (:19-69) and computeRowVariances (:72-122): per-row 256 strided partials,
 * warp shuffle tree, 8-warp sum, host row sums.  Columns beyond
 * 256*floor(width/256) are ignored. */
float ho_stddev_f32(const float *data, int width, int height, size_t stride,
                    float *mean_out);
float ho_stddev_f16(const uint16_t *data, int width, int height, size_t stride,
                    float *mean_out);

/* median_filter (median_filter.cpp:38-83): odd window, bubble-sort median,
 * edges copied from the nearest filtered value; returns the output mean. */
float ho_median_filter(const float *in, float *out, int size, int window);

/* --------------------------------------------------------------- flagger */
typedef struct {
  int tscrunch, fscrunch, nits;
  float thresh;
} ho_scrunch; /* definitions.h:76-81 */

typedef struct {
  float spec_min, spec_max; /* SPEC_MIN / SPEC_MAX, defaults -0.05 / 0.15 */
  int flag1, flag2;         /* FLAG1 / FLAG2 channel range (scrunch path) */
  int nscrunch;
  const ho_scrunch *scrunches;
  int bp_median;            /* NMEDFILT (definitions.h:39): odd window of the
                               bandpass median filter; 0 or 1 = identity */
} ho_flag_params;

/* Intermediate values of one beam's flagging, for stage-level checks. */
typedef struct {
  float bp1[8192];   /* bandpass of the raw gulp (bandpass_flag step 1) */
  float mean1, std1; /* statistics of the bandpass-corrected gulp */
  float bp2[8192];   /* bandpass after normalisation (spectral flag) */
  float bp3[8192];   /* bandpass in the final fixed scrunch */
  float mean2, std2; /* statistics after the time-series correction */
} ho_flag_trace;

/* fast_flagger for one beam (flagger.cu:345-411, NBATCH=1):
 * transpose_input -> bandpass_flag -> user scrunches -> apply_scrunch(8,8,
 * 100, flag=0, ts=1) -> transpose_output.  gulp: u8 [w][nchan];
 * out: u8 [w][nchan] (the tail of the beam's ring); ts_out: [w] or NULL;
 * flagspec: [nchan] accumulated flag fractions (scrunch path) or NULL;
 * trace may be NULL.  nchan <= 8192, w % 32 == 0, nchan % 32 == 0. */
/* As ho_flag_beam from an fp16 channel-major gulp [nchan][w] (the DADA
 * input path, transpose.cu:87-90). */
void ho_flag_beam_f16(const uint16_t *ft, int w, int nchan, const ho_flag_params *fp,
                      uint8_t *out, float *ts_out, float *flagspec, ho_flag_trace *tr);
void ho_flag_beam(const uint8_t *gulp, int w, int nchan,
                  const ho_flag_params *fp, uint8_t *out, float *ts_out,
                  float *flagspec, ho_flag_trace *trace);

/* The SCRUNCH box filter alone (convolution.cu:20-55): fp16 planes as bit
 * patterns [nchan][w], an xw x yw box of taps k. */
void ho_box_filter(const uint16_t *in, uint16_t *out, int nchan, int w, int xw,
                   int yw, float k);

/* ------------------------------------------------------------- smoothing
 * smooth.cpp:21-127.  Taps: the reference's 3 x (2sm+1) kernel, computed
 * exactly as smooth.cpp:47-58 (double u, float v, float products, float
 * normalising sum).  Returns the tap count per row (2sm+1). */
int ho_smooth_taps(int sm, float *taps3);

/* One smoothing width over a dedispersed plane dd [ndms][ntime_dd] (row
 * stride dd_stride floats), cropped as smooth.cpp:76-84 to
 * out [ndms-2][ntime_out] (row stride out_stride).
 * Arithmetic (defined here, the GPU kernel follows it):
 *   y[r][x] = fmaf(0.3f, dd[r][x] + dd[r+2][x], dd[r+1][x])   (exact sum)
 *   out[r][j] = sequential fmaf over k = 0..2sm of taps_mid[k] *
 *               y[r][clamp(j + wmax/2 + k - shift)]
 * with taps_mid the middle row of the 3-row kernel (the DM weights
 * 0.3/1/0.3 factor out), replicate borders, and shift = 0 for a kernel
 * anchored at its first tap (2sm for one anchored at its last tap). */
void ho_smooth_plane(const float *dd, int ndms, int ntime_dd, size_t dd_stride,
                     int sm, int wmax, int shift, float *out, int ntime_out,
                     size_t out_stride);

/* ho_smooth_plane with the 3 x (2sm+1) kernel applied directly (every tap
 * of every row: kernel rows outer, columns inner, one fmaf per tap) instead
 * of the factored form; the arithmetic of the emulator's NPP stand-in. */
void ho_smooth_plane_direct(const float *dd, int ndms, int ntime_dd,
                            size_t dd_stride, int sm, int wmax, int shift,
                            float *out, int ntime_out, size_t out_stride);

/* smooth(p, scale=1): every width sm = wmin*2^k < wmax, then per-width
 * (x + (-mean)) * (1/std) unless std <= 0.  boxes: [nbox][ndms-2][ntime_out]
 * packed.  mean/std: [nbox] (pre-normalisation statistics).  anchor 1: the
 * kernel's last tap sits on the output sample, which is where
 * nppiFilterBorder_32f_C1R places the reference's oAnchor {0,1} (an impulse
 * response measured on a GB300); 0: its first tap.  Returns nbox. */
int ho_smooth_normalise(const float *dd, int ndms, int ntime_dd,
                        size_t dd_stride, int wmin, int wmax, int anchor,
                        int ntime_out, float *boxes, float *mean, float *std);
/* As ho_smooth_normalise; direct != 0 uses ho_smooth_plane_direct. */
int ho_smooth_normalise_arith(const float *dd, int ndms, int ntime_dd,
                              size_t dd_stride, int wmin, int wmax, int anchor,
                              int ntime_out, float *boxes, float *mean,
                              float *std, int direct);

/* ----------------------------------------------------------------- peaks */
typedef struct {
  int32_t beam, dm_idx, width, samp;
  float snr;
} ho_cand;

/* find_peaks (peaks.cu:31-117): sigma of normalised width 0 gates the beam
 * (0.1 < sigma < 5); every sample above snr*sigma, width-major then DM row
 * then time, until `cap` candidates.  Returns the number written; *sigma0
 * receives the gate value. */
/* As ho_find_peaks; gate = 0 skips the sigma0 gate (DEBUG_ALWAYS_FIND_PEAKS). */
int ho_find_peaks_gate(const float *boxes, int nbox, int ndms, int ntime_out,
                       float snr, int beam, int cap, ho_cand *out, float *sigma0,
                       int gate);
int ho_find_peaks(const float *boxes, int nbox, int ndms, int ntime_out,
                  float snr, int beam, int cap, ho_cand *out, float *sigma0);

/* ------------------------------------------------------------ the search
 * Search parameters of one pipeline (the config keys parsed at
 * casm_hella_refactored.cu:72-169 plus the band made runtime). */
typedef struct {
  int nchan, nbeam, gulp;
  double tsamp_s;  /* data sample time */
  double plan_dt;  /* dt handed to the dedisp plan (reference: 1e-3) */
  double f0_mhz;   /* channel 0 (highest) frequency */
  double df_mhz;   /* channel width (sign ignored: descending band) */
  float dm_min, dm_max, dm_tol;
  float ti_us;     /* pulse width for the DM list (reference: 40) */
  int wmin, wmax;
  float snr;
  int max_giants;  /* MAX_GIANTS = 10000 */
  int smooth_anchor;
  ho_flag_params flag;
  int always_find_peaks; /* DEBUG_ALWAYS_FIND_PEAKS (definitions.h:66): skip the sigma0 gate */
} ho_params;

typedef struct ho_pipeline ho_pipeline;

ho_pipeline *ho_pipeline_create(const ho_params *p);
void ho_pipeline_destroy(ho_pipeline *pl);
/* Derived sizes (casm_hella_refactored.cu:184-224). */
int ho_pipeline_info(const ho_pipeline *pl, int *ntime, int *ndms,
                     int *max_delay, int *ntime_dd, int *nbox, int *min_gulp);
const float *ho_pipeline_dms(const ho_pipeline *pl);
const int32_t *ho_pipeline_delays(const ho_pipeline *pl);
/* One pass of the gulp loop (casm_hella_refactored.cu:659-835): flag all
 * beams into the rings, search beams in order while fewer than max_giants
 * candidates exist (once the ring is full), then rewind.  gulp: u8
 * [nbeam][gulp][nchan].  Returns the candidate count; *searched is 1 when
 * the search ran. */
int ho_pipeline_gulp_f16(ho_pipeline *pl, const uint16_t *gulp, ho_cand *cands,
                         int max_cands, int *searched);
int ho_pipeline_gulp(ho_pipeline *pl, const uint8_t *gulp, ho_cand *cands,
                     int max_cands, int *searched);
/* Access to the last gulp's state for stage-level checks. */
const uint8_t *ho_pipeline_ring(const ho_pipeline *pl, int beam); /* [NTIME][nchan] */
const float *ho_pipeline_flagspec(const ho_pipeline *pl);
/* Beam `beam`'s dedispersion killmask (killmask[c] == 0 drops channel c;
 * NULL: every channel); -1 for a beam outside the pipeline. */
int ho_pipeline_set_killmask(ho_pipeline *pl, int beam, const int32_t *killmask);

/* Search one window (dedisperse + smooth + find_peaks) of one beam:
 * window u8 [ntime][nchan] with ntime >= ntime_dd + max_delay. */
int ho_search_window(const ho_pipeline *pl, const uint8_t *window, int beam,
                     int cap, ho_cand *cands, float *dd_out, float *boxes_out,
                     float *mean_out, float *std_out, float *sigma0);

/* Threads used by the parallel loops (OpenMP). */
void ho_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
