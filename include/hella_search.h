/*
 * hella_search.h -- casm-hella's per-gulp FRB search stages on GB300.
 *
 * Replaces the stage functions of Coherent-All-Sky-Monitor/casm-hella that
 * the gulp loop (src/apps/casm_hella_refactored.cu:659-835) calls, over an
 * opaque context instead of the monolithic pinfo_t (src/hella/
 * definitions.h:84-173):
 *
 *   hella_create / hella_destroy   initialize (casm_hella_refactored.cu:54-309)
 *                                  / deallocator (:312-335)
 *   hella_load_gulp                H2D copy of a gulp (:688-695)
 *   hella_fast_flagger             fast_flagger   src/hella/flagger.h:75
 *   hella_dedisperse               dedisperse     src/hella/dedisperse.h:17
 *   hella_smooth                   smooth         src/hella/smooth.h:16
 *   hella_find_peaks               find_peaks     src/hella/peaks.h:17
 *   hella_clear_peaks              clear_peaks    src/hella/peaks.h:20
 *   hella_rewind                   ring rewind    (:775-797)
 *   hella_process_gulp             one pass of the loop body (:659-835)
 *
 * Every call returns a hella_status; CUDA and argument errors come back as
 * codes instead of exit() (macros.h:14-28).  All device work runs on the
 * context's stream.  A context is not thread-safe.
 */
#ifndef HELLA_SEARCH_H
#define HELLA_SEARCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hella_ctx hella_ctx;

typedef enum {
  HELLA_OK = 0,
  HELLA_ERR_INVALID_ARG = 1,  /* a parameter is out of range */
  HELLA_ERR_ALLOC = 2,        /* device or pinned host allocation failed */
  HELLA_ERR_CUDA = 3,         /* a CUDA call failed (context left usable) */
  HELLA_ERR_STATE = 4,        /* stage called out of order */
  HELLA_ERR_DEDISP = 5,       /* the dedispersion plan rejected the call */
  HELLA_ERR_BUDGET = 6,       /* HBM budget would be exceeded */
  HELLA_ERR_TIMEOUT = 7,      /* a bounded device wait expired */
  HELLA_ERR_IO = 8            /* a socket could not be opened, connected or written */
} hella_status;

#define HELLA_MAX_SCRUNCH 16
#define HELLA_MAX_GIANTS 10000 /* definitions.h:49 */

/* One SCRUNCH line "t f thresh nits" (definitions.h:76-81). */
typedef struct {
  int tscrunch, fscrunch, nits;
  float thresh;
} hella_scrunch;

/* Search configuration: the config keys of casm_hella_refactored.cu:72-169,
 * with the band (nchan, tsamp, f0, df) made runtime. */
typedef struct {
  int nchan;        /* NCHAN (definitions.h:44 fixes 3072) */
  int nbeam;        /* NBEAM */
  int gulp;         /* GULP, samples; a multiple of 32 */
  double tsamp;     /* data sample time, s */
  double plan_dt;   /* dt of the dedispersion plan (reference: 1e-3) */
  double f0_mhz;    /* frequency of channel 0 (CHAN0_FREQ) */
  double df_mhz;    /* channel width (FREQ_CHANNEL_WIDTH) */
  float dm_min, dm_max, dm_tol; /* DM_MIN, DM_MAX, DM_TOL (default 1.3) */
  float ti_us;      /* pulse width for the DM list (reference: 40) */
  int width_min, width_max;     /* WIDTH_MIN, WIDTH_MAX */
  float snr;        /* SNR */
  float spec_min, spec_max;     /* SPEC_MIN / SPEC_MAX (-0.05 / 0.15) */
  int flag1, flag2;             /* FLAG1 / FLAG2 (-1 / -1) */
  int nscrunch;                 /* SCRUNCH entries (each: flag with a tscrunch x
                                   fscrunch box at thresh; widths 1..64) */
  hella_scrunch scrunch[HELLA_MAX_SCRUNCH];
  int max_giants;   /* candidate cap per gulp (MAX_GIANTS) */
  int beam0;        /* BEAM0, added to reported beam indices */
  int smooth_anchor;/* where the 2sm+1 smoothing taps sit relative to output
                       sample x: 1 (default) inputs x-2sm..x, which is where
                       nppiFilterBorder_32f_C1R places the reference's
                       oAnchor {0,1} (smooth.cpp:54); 0: inputs x..x+2sm */
  int device;       /* GPU */
  size_t hbm_budget;/* 0 = unlimited; otherwise creation fails with
                       HELLA_ERR_BUDGET if the context would need more */
  int autotune;     /* 1: hella_create times dedispersion tile shapes on the
                       context's own buffers and keeps the fastest */
  int input_format; /* HELLA_INPUT_U8_TF (0, default): u8 [nbeam][gulp][nchan]
                       filterbank gulps; HELLA_INPUT_F16_FT (1): fp16
                       [nbeam][nchan][gulp], the DADA input (INPUT DADA,
                       casm_hella_refactored.cu:78, transpose.cu:87-90) */
  int bp_median;    /* NMEDFILT (definitions.h:39): odd window of the median
                       filter every bandpass correction applies to the
                       bandpass before dividing by it (med_filter_bandpass,
                       median_filter.cpp:85-107); 1 (the reference's value,
                       the default) is the identity; at most 63 and below
                       nchan */
  int always_find_peaks; /* DEBUG_ALWAYS_FIND_PEAKS (definitions.h:66,
                       peaks.cu:60): 1 searches for peaks whatever the
                       width-0 deviation; 0 (the reference's value, the
                       default) only when 0.1 < sigma0 < 5 */
} hella_params;

#define HELLA_INPUT_U8_TF 0
#define HELLA_INPUT_F16_FT 1

/* Dedispersion tile shape (no counterpart in the reference, whose dedisp
 * library fixes its own).  Every shape computes the same exact sums. */
typedef struct {
  int dm_per_block;       /* DM trials per tile: 16, 8, 4, 2, 1; 0 = largest
                             whose staging fits two blocks per SM */
  int samples_per_thread; /* 4: fixed by the packed ring (reported only) */
  int chan_chunk;         /* channels per staging step: 8 or 16 */
  int stages;             /* staging buffers in flight: 2..4; 0 = deepest
                             that fits two blocks per SM */
  int group;              /* DM tiles walked together per time tile (L2) */
  int add_mode;           /* 0: three-input adds; 1: load addresses as
                             multiply-adds (FMA pipe); 2: 1 + odd lanes too;
                             3: odd lanes as multiply-adds, addresses as
                             two-input adds (1-3 need dm_per_block >= 8);
                             4: sums of four adjacent channels built once
                             per delay pattern of a 16-trial tile and shared
                             by its trials (dm_per_block 0 or 16; chan_chunk
                             and the per-beam killmask tables unused);
                             5: pair rows -- adjacent active channels summed
                             once per window and relative delay into rows
                             in device memory, then summed by 16-trial tiles
                             (dm_per_block 0 or 16; chan_chunk/2 pairs per
                             stage; the batched context builds and sums the
                             beams one after another in one row buffer);
                             6: as 5 with rows of four channels (about 3x
                             the rows, half the shared-memory reads).  The
                             rows (mode 5: about 5.8 GB for 2048 channels,
                             DM 0-2000, gulp 65536; mode 6: 19 GB) are held
                             while the mode is set and count against
                             hbm_budget (HELLA_ERR_BUDGET) */
} hella_tuning;

/* Derived sizes (casm_hella_refactored.cu:184-224). */
typedef struct {
  int ntime;        /* NTIME: gulp + max_delay + width_max rounded up */
  int ndms;         /* DM trials */
  int max_delay;    /* samples */
  int ntime_dd;     /* gulp + width_max: dedispersed samples kept */
  int ntime_out;    /* gulp */
  int nboxcar;      /* smoothing widths width_min*2^k < width_max */
  int min_gulp;     /* first gulp index that is searched */
  int gulp_index;   /* gulps processed so far */
  size_t device_bytes; /* device memory held by the context */
} hella_info;

/* One candidate: a sample above SNR x sigma (peaks.cu:232-242). */
typedef struct {
  int32_t beam;     /* beam index + beam0 */
  int32_t dm_idx;   /* DM trial (row + 1 of the smoothed plane) */
  int32_t width;    /* smoothing width index */
  int32_t samp;     /* sample within the gulp's output window */
  float snr;        /* normalised smoothed value */
} hella_cand;

void hella_params_default(hella_params *p);
hella_status hella_create(hella_ctx **ctx, const hella_params *p);
void hella_destroy(hella_ctx *ctx);
hella_status hella_set_stream(hella_ctx *ctx, void *stream);
hella_status hella_get_info(const hella_ctx *ctx, hella_info *info);
/* DM of each trial (host memory owned by the context). */
const float *hella_get_dm_list(const hella_ctx *ctx);
/* Killmask shared by all beams (0 = channel dropped from dedispersion). */
hella_status hella_set_killmask(hella_ctx *ctx, const int *killmask);

/* Gulp input: u8 [nbeam][gulp][nchan] (time-major, as a SIGPROC gulp), or
 * fp16 [nbeam][nchan][gulp] with input_format HELLA_INPUT_F16_FT;
 * on_device != 0 means `gulp` is a device pointer. */
hella_status hella_load_gulp(hella_ctx *ctx, const uint8_t *gulp,
                             int on_device);
hella_status hella_fast_flagger(hella_ctx *ctx);
hella_status hella_dedisperse(hella_ctx *ctx, int beam);
hella_status hella_smooth(hella_ctx *ctx, int scale);
hella_status hella_find_peaks(hella_ctx *ctx, int beam);
hella_status hella_clear_peaks(hella_ctx *ctx);
hella_status hella_rewind(hella_ctx *ctx);
/* Candidates gathered since the last clear (host copy). */
hella_status hella_get_peaks(hella_ctx *ctx, hella_cand *out, int max,
                             int *n);
/* Load + flag + (search every beam while under max_giants, once the ring
 * is full) + rewind.  *searched is set to 1 when the search ran. */
hella_status hella_process_gulp(hella_ctx *ctx, const uint8_t *gulp,
                                int on_device, hella_cand *out, int max,
                                int *n, int *searched);

/* Tile shape of the context's dedispersion (see hella_tuning). */
hella_status hella_get_tuning(const hella_ctx *ctx, hella_tuning *t);
hella_status hella_set_tuning(hella_ctx *ctx, const hella_tuning *t);
/* Times one dedispersion of the context's ring with shape t (the current
 * shape if t is NULL): best of `reps` runs, milliseconds.  Overwrites the
 * dedispersed plane; call between gulps.  Synchronous. */
hella_status hella_time_dedisp(hella_ctx *ctx, const hella_tuning *t, int reps,
                               float *ms);
/* Coordinate search over the tile shape, keeping the fastest; *best and
 * *best_ms (may be NULL) receive it.  Call between gulps.  Synchronous. */
hella_status hella_autotune(hella_ctx *ctx, int reps, hella_tuning *best,
                            float *best_ms);

/* Inspection (host copies, synchronous). */
/* The beam's search window, u8 [ntime][nchan] time-major, oldest first. */
hella_status hella_copy_window(hella_ctx *ctx, int beam, uint8_t *out);
/* Last dedispersed plane, fp32 [ndms][ntime_dd]. */
hella_status hella_copy_dedisp(hella_ctx *ctx, float *out);
/* Last normalised smoothed planes, fp32 [nboxcar][ndms-2][ntime_out]. */
hella_status hella_copy_boxes(hella_ctx *ctx, float *out);
/* Per-width mean/std before normalisation and the peak gate sigma. */
hella_status hella_get_smooth_stats(hella_ctx *ctx, float *mean,
                                    float *std, float *sigma0);
/* Flagger statistics of a beam's last gulp: bp1/bp2/bp3 [nchan] and
 * scalars[4] = {mean1, std1, mean2, std2}; any pointer may be NULL. */
hella_status hella_get_flag_stats(hella_ctx *ctx, int beam, float *bp1,
                                  float *bp2, float *bp3, float *scalars,
                                  float *ts);
/* Accumulated per-channel flag fractions (d_flagSpec, flagger.cu:334). */
hella_status hella_get_flag_spec(hella_ctx *ctx, float *out);

/* ---- Batched multi-beam search (no counterpart in the reference, whose
 * gulp loop runs the stages beam after beam).  Every stage runs for all
 * beams in one launch per pass; the per-gulp launches are captured once in a
 * CUDA graph and replayed.  Beam b has its own DM ceiling and killmask, and
 * its candidates are those of a single-beam context created with
 * dm_max = dm_max[b] and that killmask, fed the same gulps. */
typedef struct hella_batch hella_batch;

typedef struct {
  hella_params base;     /* base.nbeam beams; base.dm_max is ignored when
                            dm_max is given; base.max_giants caps each beam */
  const float *dm_max;   /* [nbeam] DM ceiling of each beam, or NULL */
  const int *killmask;   /* [nbeam][nchan], 0 = channel dropped, or NULL */
  int widths_per_pass;   /* smoothing widths held in HBM at once; 0: as
                            many as base.hbm_budget (or free memory) allows */
  int use_graph;         /* 1: capture the per-gulp launches in a CUDA graph */
  int dynamic;           /* 1: beams are slots that join and leave (each sized
                            for base.dm_max); 0: fixed beams, exact sizes */
  const int *member;     /* [nbeam] 1 = slot in use at creation (NULL: all) */
  int inflight;          /* gulps in flight for submit/poll: 1 or 2 */
  float bp_alpha;        /* weight of the newest gulp in the running
                            (exponentially weighted) bandpass, 0 < a <= 1 */
} hella_batch_params;

void hella_batch_params_default(hella_batch_params *p);
hella_status hella_batch_create(hella_batch **b, const hella_batch_params *p);
void hella_batch_destroy(hella_batch *b);
/* Stream of the batch's device work (a cudaStream_t other than the legacy
 * default stream, which cannot be captured; NULL: the batch's own stream). */
hella_status hella_batch_set_stream(hella_batch *b, void *stream);
/* Sizes of beam `beam` (as hella_get_info of its single-beam context). */
hella_status hella_batch_get_info(const hella_batch *b, int beam, hella_info *info);
/* One gulp u8 [nbeam][gulp][nchan] of every beam: flag, dedisperse, smooth
 * and find peaks for all beams.  out receives min(total, max) candidates,
 * beam by beam, each beam's in the single-beam order; counts[b] (may be
 * NULL) the number of beam b, searched[b] (may be NULL) whether beam b was
 * searched.  *n = candidates written to out. */
hella_status hella_batch_process_gulp(hella_batch *b, const uint8_t *gulp, int on_device,
                                      hella_cand *out, int max, int *n, int *counts,
                                      int *searched);
/* Streaming (config keys of the serving loop; no counterpart in the
 * reference).  submit enqueues one gulp (u8 [nbeam][gulp][nchan]; a host
 * buffer must stay valid until its result is polled, and is best pinned):
 * its copy to the device overlaps the search of the gulp before it.  poll
 * returns the oldest submitted gulp's results, blocking until they are
 * ready; latency_ms (may be NULL) receives the host time from submit to
 * results, device_ms the device time of its search.  HELLA_ERR_STATE: no
 * free in-flight buffer (submit) or nothing submitted (poll). */
hella_status hella_batch_submit(hella_batch *b, const uint8_t *gulp, int on_device);
hella_status hella_batch_poll(hella_batch *b, hella_cand *out, int max, int *n, int *counts,
                              int *searched, float *latency_ms, float *device_ms);
/* Slot `beam` joins (member = 1, with its DM ceiling and killmask
 * [nchan] or NULL) or leaves (member = 0) from the next submitted gulp on;
 * a joining slot starts as a fresh single-beam context would (its window is
 * searched once it holds only its own samples).  Dynamic batches only; no
 * gulp may be in flight.  dm_max above the batch's base.dm_max:
 * HELLA_ERR_BUDGET. */
hella_status hella_batch_set_beam(hella_batch *b, int beam, int member, float dm_max,
                                  const int *killmask);
/* Running bandpass of a slot: per channel, the exponentially weighted mean
 * (weight bp_alpha for the newest gulp) of calc_bandpass_new over the gulps
 * since the slot joined; fp32 [nchan]. */
hella_status hella_batch_get_bandpass(hella_batch *b, int beam, float *out);
/* Accumulated per-channel flag fractions of the SCRUNCH entries over all
 * beams and gulps (d_flagSpec, flagger.cu:333-334), fp32 [nchan]. */
hella_status hella_batch_get_flag_spec(hella_batch *b, float *out);
/* Device bytes a batch with these parameters would hold (admission by HBM
 * budget: size nbeam so that this stays within the budget). */
hella_status hella_batch_bytes(const hella_batch_params *p, size_t *bytes);

/* Inspection: beam's last dedispersed plane, fp32 [ndms_b][ntime_dd]. */
hella_status hella_batch_copy_dedisp(hella_batch *b, int beam, float *out);
hella_status hella_batch_get_tuning(const hella_batch *b, hella_tuning *t);
hella_status hella_batch_set_tuning(hella_batch *b, const hella_tuning *t);
/* Times the all-beam dedispersion launch with shape t (NULL: current). */
hella_status hella_batch_time_dedisp(hella_batch *b, const hella_tuning *t, int reps,
                                     float *ms);
hella_status hella_batch_autotune(hella_batch *b, int reps, hella_tuning *best,
                                  float *best_ms);
/* Kernel launches in the captured per-gulp graph (HELLA_ERR_STATE before
 * the first graph gulp). */
hella_status hella_batch_graph_kernels(const hella_batch *b, int *kernels);
/* Per-gulp device time of the last processed gulp's stages, ms:
 * [0] whole gulp (graph), recorded with CUDA events. */
hella_status hella_batch_last_gulp_ms(const hella_batch *b, float *ms);

const char *hella_status_string(hella_status s);

/* Device self-check of the fp16 arithmetic the flagger relies on (no
 * counterpart in the reference, whose kernels simply call these
 * intrinsics): over every pair of positive finite binary16 values, counts
 * the cases where __hdiv differs from the correctly rounded quotient
 * (fp32 IEEE division rounded once to fp16), and likewise __hadd/__hmul on
 * a strided subset.  first_bad receives (a << 16 | b) of the first
 * mismatch.  Synchronous. */
hella_status hella_fp16_selftest(int device, unsigned long long *mismatches,
                                 uint32_t *first_bad);

/* Measurement helpers (no counterpart in the reference).
 * hella_int_add_peak: 32-bit integer adds per second the device sustains
 * from registers (independent add chains on every SM, timed with CUDA
 * events); the dedispersion roofline's denominator.  Synchronous.
 * hella_kernel_launches: kernels this library has launched in this process. */
hella_status hella_int_add_peak(int device, double *adds_per_s);
/* hella_smem_read_peak: shared-memory bytes per second the device's SMs
 * read with conflict-free 16-byte loads (all SMs, measured), the ceiling of
 * add mode 5's summing kernel, which reads one byte per channel-sample. */
hella_status hella_smem_read_peak(int device, double *bytes_per_s);
unsigned long long hella_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
