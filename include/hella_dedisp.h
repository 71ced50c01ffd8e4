/*
 * hella_dedisp.h -- brute-force direct dedispersion on GB300 (sm_103a),
 * with the plan/execute interface casm-hella drives through the dedisp
 * library.  The function set mirrors that interface one for one under the
 * `hdd_` prefix, so a caller swaps `dedisp_` for `hdd_` and links
 * libhella_gb300.so.  Reference call sites replaced (Coherent-All-Sky-
 * Monitor/casm-hella):
 *   src/apps/casm_hella_refactored.cu:205   dedisp_create_plan
 *   src/apps/casm_hella_refactored.cu:207   dedisp_generate_dm_list
 *   src/apps/casm_hella_refactored.cu:208   dedisp_get_dm_list
 *   src/apps/casm_hella_refactored.cu:209   dedisp_get_dm_count
 *   src/apps/casm_hella_refactored.cu:210   dedisp_get_max_delay
 *   src/hella/src/dedisperse.cpp:32-38       dedisp_execute_adv
 *   src/hella/src/dedisperse.cpp:50-91       error names (dedisp_error)
 *
 * Conventions (the dedisp library is not part of the reference; these are
 * this library's definitions, restated from the published method):
 *   - channel 0 is the highest frequency f0; channel c is f0 - c*|df| (MHz);
 *   - delay(c, DM) = (int)(DM * tab[c] + 0.5f) in fp32, with
 *     tab[c] = 4.148808e3 (1/f_c^2 - 1/f0^2) / dt samples per unit DM;
 *   - the DM list follows the Cordes & McLaughlin smearing tolerance;
 *   - out_nbits = 32 writes each sum as the exact integer in fp32;
 *   - in_nbits = 8: unsigned bytes, time-major, in_stride bytes per sample.
 * Every call returns a status; nothing exits or throws.  One plan per
 * thread; all device work is issued on the plan's stream.
 */
#ifndef HELLA_DEDISP_H
#define HELLA_DEDISP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hdd_plan_struct *hdd_plan;
typedef unsigned long hdd_size;
typedef float hdd_float;
typedef unsigned char hdd_byte;
typedef int hdd_bool;

/* Same order and meaning as the names at dedisperse.cpp:54-88. */
typedef enum {
  HDD_NO_ERROR = 0,
  HDD_MEM_ALLOC_FAILED,
  HDD_MEM_COPY_FAILED,
  HDD_NCHANS_EXCEEDS_LIMIT,
  HDD_INVALID_PLAN,
  HDD_INVALID_POINTER,
  HDD_INVALID_STRIDE,
  HDD_NO_DM_LIST_SET,
  HDD_TOO_FEW_NSAMPS,
  HDD_INVALID_FLAG_COMBINATION,
  HDD_UNSUPPORTED_IN_NBITS,
  HDD_UNSUPPORTED_OUT_NBITS,
  HDD_INVALID_DEVICE_INDEX,
  HDD_DEVICE_ALREADY_SET,
  HDD_PRIOR_GPU_ERROR,
  HDD_INTERNAL_GPU_ERROR,
  HDD_UNKNOWN_ERROR,
  HDD_STATIC_SCRATCH_EXCEEDED /* hdd_execute_noalloc: needs more than its
                                 fixed scratch (HDD_NOALLOC_SCRATCH_BYTES) */
} hdd_error;

/* Execute flags; the reference passes 1<<2 (device pointers,
 * dedisperse.cpp:32-38). */
#define HDD_USE_DEFAULT 0
#define HDD_HOST_POINTERS (1 << 1)
#define HDD_DEVICE_POINTERS (1 << 2)
#define HDD_WAIT (1 << 3)
#define HDD_ASYNC (1 << 4)

#define HDD_MAX_NCHANS 16384

/* dedisp_create_plan (casm_hella_refactored.cu:205): nchans channels of
 * width df (MHz, sign ignored) below f0 (MHz), samples of dt seconds. */
hdd_error hdd_create_plan(hdd_plan *plan, hdd_size nchans, hdd_float dt,
                          hdd_float f0, hdd_float df);
void hdd_destroy_plan(hdd_plan plan);

/* Selects the CUDA device for plans created afterwards on this thread. */
hdd_error hdd_set_device(int device_idx);
/* Stream (a cudaStream_t passed as void*) for the plan's device work;
 * NULL selects the legacy default stream. */
hdd_error hdd_set_stream(hdd_plan plan, void *stream);

hdd_error hdd_set_dm_list(hdd_plan plan, const hdd_float *dm_list,
                          hdd_size count);
/* dedisp_generate_dm_list (casm_hella_refactored.cu:207): trials from
 * dm_start until >= dm_end for a pulse of width ti (microseconds) and
 * smearing tolerance tol. */
hdd_error hdd_generate_dm_list(hdd_plan plan, hdd_float dm_start,
                               hdd_float dm_end, hdd_float ti, hdd_float tol);
/* killmask[c] == 0 drops channel c from every sum. */
hdd_error hdd_set_killmask(hdd_plan plan, const hdd_bool *killmask);
/* hdd_set_pair_rows -- no counterpart in the reference.  channels = 2 (or
 * 1): the execute calls dedisperse from pair rows (adjacent active channels
 * summed once per call and relative delay into rows in device memory, then
 * summed by 16-trial tiles); 4: from rows of four channels; 0: channel by
 * channel (the default); anything else: HDD_UNKNOWN_ERROR.  The same sums,
 * about 1.5x (pairs) to 1.7x (quads) faster on long DM lists, for the rows'
 * device memory (pairs: about 5.8 GB for 2048 channels, DM 0-2000, 66048
 * output samples; quads about 3x that), which the plan holds until the mode
 * is switched off or the plan is destroyed.  A DM list whose stages do not
 * fit shared memory falls back to the channel-by-channel kernel; a failed
 * allocation returns HDD_MEM_ALLOC_FAILED.  hdd_execute_noalloc does not
 * use it. */
hdd_error hdd_set_pair_rows(hdd_plan plan, int channels);
/* hdd_get_pair_tables -- no counterpart in the reference; for tests.  Host
 * copies of the group-row tables the plan builds for trials [first_dm_idx,
 * first_dm_idx + dm_count), `channels` (2 or 4) a group, stage_groups (4
 * or 8) groups a stage and time_tiles tiles of 1024 output samples, as the
 * execute calls would use them.  The pointers stay valid until the plan's
 * tables change.  Word i of row r (group k) holds, for the window position
 * p = first + (i / stride) * 1024 + i % stride (first = rinfo[r][3],
 * stride = rtile[r]), x[c0][p] + sum_i x[c_i][p + r_i] in its low 16 bits
 * and the same at p + 512 in the high bits; a stage record is
 * {groups, rows, 0, 0}, then stage_groups x 16 trial byte offsets into the
 * staged rows, then 32 x {first word of time tile 0 (low, high 32 bits),
 * words | byte slot / 16 << 16, the row's words per time tile}. */
typedef struct {
  int channels, stage_groups, time_tiles, ntiles, ngroups, nrows, nrec, rec_ints;
  int max_stage_bytes, max_span;
  long npos, words;
  const int *rinfo;       /* [nrows][4] c0, c1 (-1: none), r1, position of word 0 */
  const int *rinfo2;      /* [nrows][4] c2, c3 (-1: none), r2, r3 */
  const long long *roff;  /* [nrows] first word of the row */
  const int *rwords;      /* [nrows] words of the row */
  const int *rtile;       /* [nrows] words per time tile (1024: one run) */
  const int *prow;        /* [ngroups + 1] first row of each group */
  const int *prange;      /* [ngroups][3][2] smallest, largest r_i */
  const int *rec;         /* [nrec][rec_ints] stage records */
  const int *tile_st;     /* [ntiles + 1] first record of each 16-trial tile */
} hdd_pair_tables_view;
hdd_error hdd_get_pair_tables(hdd_plan plan, hdd_size first_dm_idx, hdd_size dm_count, int channels,
                              int stage_groups, int time_tiles, hdd_pair_tables_view *out);

hdd_size hdd_get_max_delay(const hdd_plan plan);
hdd_size hdd_get_dm_delay(const hdd_plan plan, int dm_trial);
hdd_size hdd_get_channel_count(const hdd_plan plan);
hdd_size hdd_get_dm_count(const hdd_plan plan);
const hdd_float *hdd_get_dm_list(const hdd_plan plan);
const hdd_bool *hdd_get_killmask(const hdd_plan plan);
hdd_float hdd_get_dt(const hdd_plan plan);
hdd_float hdd_get_df(const hdd_plan plan);
hdd_float hdd_get_f0(const hdd_plan plan);
/* Host copy of the integer delay table, [dm_count][nchans]. */
const int *hdd_get_delay_table(const hdd_plan plan);

/* out[d][t] for t < nsamps - max_delay (dedisp_execute). */
hdd_error hdd_execute(hdd_plan plan, hdd_size nsamps, const hdd_byte *in,
                      hdd_size in_nbits, hdd_byte *out, hdd_size out_nbits,
                      unsigned flags);
/* dedisp_execute_adv (dedisperse.cpp:32-38): strides in bytes. */
hdd_error hdd_execute_adv(hdd_plan plan, hdd_size nsamps, const hdd_byte *in,
                          hdd_size in_nbits, hdd_size in_stride,
                          hdd_byte *out, hdd_size out_nbits,
                          hdd_size out_stride, unsigned flags);
/* Subset of DM trials [first_dm_idx, first_dm_idx + dm_count); output row
 * 0 is trial first_dm_idx. */
hdd_error hdd_execute_guru(hdd_plan plan, hdd_size nsamps, const hdd_byte *in,
                           hdd_size in_nbits, hdd_size in_stride,
                           hdd_byte *out, hdd_size out_nbits,
                           hdd_size out_stride, hdd_size first_dm_idx,
                           hdd_size dm_count, unsigned flags);

/* Text for a status, as get_dedisp_error (dedisperse.cpp:50-91). */
const char *hdd_get_error_string(hdd_error error);

/* hdd_execute_noalloc -- no counterpart in the reference.
 *
 * hdd_execute_adv with device pointers, for callers that cannot allocate
 * device memory while they run: a real-time loop that must not stall in
 * the allocator or risk an out-of-memory failure mid-stream, code running
 * under a device-memory pool or budget owned by another component, and
 * hosts that forbid allocation after start-up.  Every buffer the other
 * execute calls allocate on demand (the channel-major staging copy, the
 * packed ring, the dedispersion tile tables) lives instead in one fixed array of
 * HDD_NOALLOC_SCRATCH_BYTES compiled into the library; every GPU that loads
 * the library holds that array until the process exits.  The call makes no
 * cudaMalloc/cudaFree and no other allocating call.
 *
 * Limits: the dedispersion tile tables (at most 32 bytes per DM trial per
 * active channel; 5 with the usual 16-trial tiles) plus 5*nchans*R bytes
 * (R = nsamps rounded up to a multiple of 4), each part aligned to 256
 * bytes, must fit in HDD_NOALLOC_SCRATCH_BYTES, else
 * HDD_STATIC_SCRATCH_EXCEEDED.  nsamps above 65535*32 returns
 * HDD_UNKNOWN_ERROR (the transpose's grid limit, as hdd_execute_guru).  in
 * and out are device pointers (HDD_HOST_POINTERS is rejected).
 *
 * Set-up: the first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current) and clears its status
 * word with a synchronous cudaMemset; make that first call before any
 * stream capture.
 *
 * Sharing: all calls share the array.  Each call overwrites the tables and
 * buffers it uses before reading them, so no data carries over from the
 * previous call; two calls whose device work overlaps in time (other
 * streams, other threads) race on it.
 *
 * Errors on the device: a staging wait that times out sets the status word,
 * which stays set until a synchronous call (no HDD_ASYNC) reads it.  That
 * call returns HDD_INTERNAL_GPU_ERROR and clears the word, so it reports a
 * timeout of its own or of any HDD_ASYNC call before it; an HDD_ASYNC call
 * itself returns HDD_NO_ERROR once its work is queued. */
#define HDD_NOALLOC_SCRATCH_BYTES (32ul << 20)
hdd_error hdd_execute_noalloc(hdd_plan plan, hdd_size nsamps,
                              const hdd_byte *in, hdd_size in_nbits,
                              hdd_size in_stride, hdd_byte *out,
                              hdd_size out_nbits, hdd_size out_stride,
                              unsigned flags);

#ifdef __cplusplus
}
#endif
#endif
