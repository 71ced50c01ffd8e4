// hg_internal.h -- shared declarations of the GB300 search library.
//
// Layout of the per-beam state in HBM (all device arrays are beam-major):
//   gulp     u8  [nbeam][gulp][nchan]       time-major input gulp
//   plain    u8  [nbeam][nchan][R]          channel-major ring, R = NTIME
//   packed   u32 [nbeam][nchan][R]          word q holds samples q, q+S,
//                                           q+2S, q+3S (S = kPackS) of the
//                                           ring, the dedispersion operand
//   lut      f16 [nbeam][nchan][256]        flagger value of each u8 level
//   dd       f32 [ndms][ntime_dd]           dedispersed sums of one beam
//   boxes    f32 [nbox][ndms-2][ntime_out]  smoothed planes (pre-normalise)
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <cstddef>
#include <cstdint>
#include <vector>

namespace hg {

// Kernels launched by this library (process-wide, for the benchmark).
void count_launches(unsigned n);

// Interleave stride of the packed ring: one 32-bit word carries the samples
// q, q+S, q+2S, q+3S of a channel, so a warp reading 32 consecutive words
// at any delay gets 4 x 32 consecutive output samples of one DM trial.
constexpr int kPackS = 256;
// Dedispersion block: kPackS threads, one per packed word position.
constexpr int kDedispThreads = kPackS;
// DM tiles walked together per time tile by the persistent dedispersion
// kernel (default; the search contexts may tune it).
constexpr int kDedispGroup = 8;

// ------------------------------------------------------------- flagger
struct FlagState {
  int nbeam, nchan, gulp;
  float spec_min, spec_max;
  float *bp1, *bp2, *bp3;   // [nbeam][nchan]
  float *part;              // [nbeam][nchan][256] reduction partials
  float *rowval;            // [nbeam][nchan] per-channel row statistic
  float *scal;              // [nbeam][8] mean1 std1 mean2 std2
  __half *hsc;              // [nbeam][8] half(-mean1) half(1/std1) ...
  __half *lut;              // [nbeam][nchan][256]
  uint8_t *flag2;           // [nbeam][nchan] spectral flag decision
  float *ts;                // [nbeam][gulp]
  __half *hts;              // [nbeam][gulp]
  // SCRUNCH entries (apply_scrunch with flag = 1, flagger.cu:271-343): the
  // data stop being a function of (channel, u8 level), so the flagger then
  // keeps fp16 planes [nbeam][nchan][gulp] (channel-major) instead
  int nscrunch;
  int sc_t[16], sc_f[16];   // time and channel widths of each entry
  float sc_thresh[16];
  int flag_lo, flag_hi;     // FLAG1 / FLAG2: channels [lo, hi) zeroed by each entry
  __half *P, *M, *S;        // data, threshold mask, box-filtered plane
  float *bpx;               // [nbeam][nchan] bandpass of an entry
  float *fsb;               // [nbeam][nchan] flag fractions of an entry
  float *flagspec;          // [nchan] flag fractions accumulated over beams and gulps
  int f16_input;            // gulps arrive as fp16 [nbeam][nchan][gulp] (DADA input):
                            // every stage then runs on the planes
  int bp_median;            // window of the bandpass median filter (1: identity)
};
// Largest bandpass median window (hella_params.bp_median).
constexpr int kMaxBpMedian = 63;
// Largest SCRUNCH widths the box filter stages in shared memory.
constexpr int kMaxScrunch = 64;

// Runs the whole parity flagger for all beams of `gulp` (u8 [nbeam][gulp]
// [nchan]) and writes the requantised output into the plain ring at ring
// position `wpos` (mod R) of every beam.
// `gulp` is u8 [nbeam][gulp][nchan], or fp16 [nbeam][nchan][gulp] when
// st.f16_input is set.
cudaError_t flag_gulp(const FlagState &st, const void *gulp, uint8_t *plain,
                      long R, long wpos, cudaStream_t s);
// As above with the ring position read on the device from pos->wpos.
cudaError_t flag_gulp_dev(const FlagState &st, const void *gulp, uint8_t *plain,
                          long R, const struct GulpPos *pos, cudaStream_t s);

// ---------------------------------------------------------- packing
// Rebuild packed words at ring positions [q0, q0 + nq) (mod R) of every
// beam from the plain ring.  keep ([nbeam][nchan], may be null): channels
// with keep == 0 are packed as zeros, which drops them from every sum.
cudaError_t pack_ring(const uint8_t *plain, uint32_t *packed, int nbeam,
                      int nchan, long R, long q0, long nq, cudaStream_t s,
                      const uint8_t *keep = nullptr);
// Rebuilds the words a gulp written at pos->wpos changed:
// [wpos - 3*kPackS, wpos + gulp) mod R.
cudaError_t pack_gulp_dev(const uint8_t *plain, uint32_t *packed, int nbeam, int nchan,
                          long R, int gulp, const struct GulpPos *pos, cudaStream_t s,
                          const uint8_t *keep);
// Time-major input [nsamps][in_stride] -> channel-major plain [nchan][R].
cudaError_t transpose_tf(const uint8_t *in, size_t in_stride, int nsamps,
                         int nchan, uint8_t *plain, long R, cudaStream_t s);

// ------------------------------------------------------ dedispersion
// One beam of a dedispersion launch.
struct DedispBeam {
  const uint32_t *packed;   // [nchan][R] packed words of the beam
  float *out;               // [dm_count][out_stride]; row i = trial dm_first + i
  long win0;                // ring position of window sample 0
  int dm_count;             // trials of this beam: the first dm_count of the table
  int item0;                // first work item of the beam (prefix over beams)
  // the beam's own tile tables over its nact channels (laid out as the
  // launch's tile_meta / tile_off); null: the launch's tables
  const int4 *meta;
  const int *off;
  int nact;
};

struct DedispArgs {
  const DedispBeam *beams;  // device array [nbeam]; null: the single beam `one`
  DedispBeam one;
  int nbeam;
  int nitems;               // work items: (beam, DM tile, time tile)
  int ntt;                  // time tiles per beam (4*kPackS samples each)
  int group;                // DM tiles walked together per time tile (L2 reuse)
  long R;                   // ring length (words per channel row), % 4 == 0
  int nact;                 // channels in the tables
  int dm_first;             // first trial of the tables
  int nout;                 // output samples per trial
  long out_stride;
  int dpt;                  // DM trials per tile (16, 8, 4, 2 or 1)
  int cc;                   // channels per pipeline stage (8 or 16)
  int nbuf;                 // staging buffers, 2..4 (0: deepest that fits)
  int mode;                 // pipe balance of the adds (0-3; 1-3 need dpt >= 8), or 4: sub-band
                            // sums of four channels per pattern (dpt 16, tables below), or
                            // 5 / 6: rows of channel pairs / quads (dpt 16, one beam a launch,
                            // pair tables below)
  int unit;                 // must be 1
  int max_spread;           // largest tile_meta spread
  const int4 *tile_meta;    // [ntiles][nact] {channel, smallest delay(c, d) of the tile, spread, 0}
  const int *tile_off;      // [ntiles][nact][max(dpt,4)] 4*(delay(c,d) - that delay), bytes
  int *err;                 // device status word: bit 0 = a staging wait timed out (may be null)
  int varied;               // some beam has tables of its own (dpt >= 8): stage counts differ
  // mode 4: per (tile, group of four channels of tile_meta) a record in sub_pool
  const int2 *sub_index;    // [ntiles][ngroups] {offset in sub_pool (ints), record bytes}
  const int *sub_pool;
  int sub_words;            // most pattern-row words of a record
  int sub_rec;              // largest record, bytes (a multiple of 16)
  // mode 5 (see PairTables): the rows are rebuilt from `one.packed` at `one.win0`
  const int4 *pair_rinfo;
  const int4 *pair_rinfo2;
  const long long *pair_roff;
  const int *pair_rwords;
  const int *pair_rtile;
  const int *pair_prow;
  const int2 *pair_prange;
  const int4 *pair_rec;
  const int *pair_tile_st;
  uint32_t *pair_rows;
  const int *pair_rend;     // [nbeam][npair] end of the rows to build per group (null: all rows)
  long pair_rows_stride;    // words between the rows of consecutive beams of the launch
  int pair_npair, pair_span, pair_stage, pair_g, pair_lanecap;
  long pair_npos;
};
// One beam's tile tables gathered from a launch's tables (all nch channels):
// rows [meta0, meta0 + ntiles * nact) of the output, channels chans[chans0 ..).
struct TableJob {
  long meta0;
  int chans0, nact, ntiles;
};
// Gathers the rows of every job's channels from meta/off (tile shape dpt >= 8)
// into bmeta / boff.
cudaError_t gather_tables(const int4 *meta, const int *off, int nch, int dpt, const TableJob *jobs, int njobs,
                          int max_tiles, const int *chans, int4 *bmeta, int *boff, cudaStream_t s);
// Work items of one beam for a tile shape.
inline int dedisp_items(int dm_count, int dpt, int ntt) { return (dm_count + dpt - 1) / dpt * ntt; }
inline int dedisp_time_tiles(int nout) { return (nout + 4 * kPackS - 1) / (4 * kPackS); }
// Launches the persistent kernel over all items of `a`.
cudaError_t dedisperse(const DedispArgs &a, cudaStream_t s);
// Shared memory of one block for a tile shape; 0 when it does not fit.
size_t dedisp_smem_bytes(int dpt, int cc, int max_spread);
// Deepest staging pipeline (2..4 buffers) of a tile shape within the
// two-blocks-per-SM budget; 0 when two buffers do not fit.
int dedisp_nbuf(int dpt, int cc, int max_spread);

// Host-side tile tables for trials [dm_first, dm_first + dm_count) over the
// active channels, for `dpt` trials per tile (dpt = 0: the largest tile
// whose double-buffered staging of cc channels fits in shared memory).
struct DedispTables {
  int dpt = 0, max_spread = 0, ntiles = 0, offw = 0;
  std::vector<int4> meta;
  std::vector<int> off;
};
DedispTables dedisp_tables(const int *delays_host, int nchan, const int *chans_host, int nact,
                           int dm_first, int dm_count, int dpt = 0, int cc = 8);
// Tables of add mode 4 (sub-band sums shared by a 16-trial tile's trials,
// groups of four consecutive active channels); meta as DedispTables.meta
// for 16-trial tiles.
constexpr int kSubG = 4;
constexpr int kSubDPT = 16;
struct SubTables {
  int ntiles = 0, ngroups = 0, max_spread = 0, max_words = 0, max_rec = 0;
  std::vector<int4> meta;
  std::vector<int2> index;
  std::vector<int> pool;
};
SubTables dedisp_sub_tables(const int *delays_host, int nchan, const int *chans_host, int nact,
                            int dm_first, int dm_count);
// Shared memory of one add-mode-4 block.
size_t dedisp_sub_smem(int max_spread, int max_words, int max_rec, int nbuf);

// Add modes 5 and 6: rows of channel groups.  The active channels are taken
// g at a time in order (g = 2, pairs, in mode 5; g = 4 in mode 6; the last
// group may be smaller).  For each group (c0, c1, ...) and each pattern of
// relative delays r_i = delay(c_i, d) - delay(c0, d) that a trial of the
// range gives it, one row holds x[c0][p] + sum_i x[c_i][p + r_i] for the
// window positions p that those trials read, two samples a word (p in the
// low and p + 512 in the high 16 bits).  The rows are rebuilt from the
// packed ring for every window (k_pair_build), after which a 16-trial tile
// sums, group by group, the row of each trial's pattern at the trial's
// delay of c0 (k_pair_sum): 1/g of the adds of the channel-by-channel sum,
// with no byte splitting in the inner loop.  A stage of a tile stages the
// windows of the rows its groups use; its record is
//   int4 {groups, rows, 0, 0}
//   int  [cc][16] byte offset, in the staged rows, of each trial's window
//   int4 [kPairRowsMax] {first word of tile 0 (low, high 32 bits),
//                        words | byte slot / 16 << 16, the row's words per time tile}
// (a copy of time tile tt starts at first word + tt x words per time tile).
constexpr int kPairDPT = 16;
constexpr int kPairRowsMax = 32;  // rows per stage: one per lane of the staging warp
constexpr int kPairGMax = 4;      // channels per group
constexpr int kPairMaxBeams = 4;  // beams one pair of launches serves (batched context)
// Groups per 16-bit lane before widening: lanecap x g x 255 < 2^16.
inline int pair_lanecap(int g) { return 65535 / (255 * g); }
__host__ __device__ constexpr int pair_rec_int4(int cc) { return 1 + cc * kPairDPT / 4 + kPairRowsMax; }
// Staged row bytes a stage of cc groups may hold (a single group may exceed it).
inline int pair_stage_budget(int cc) { return cc <= 4 ? 24 * 1024 : 36 * 1024; }
struct PairTables {
  int g = 0, cc = 0, ntt = 0, ntiles = 0, npair = 0, nrows = 0, dm_count = 0;
  int max_stage = 0;            // largest staged row bytes of a stage
  int max_span = 0;             // largest r_i range of one group and channel
  long npos = 0;                // window positions the rows cover
  long words = 0;               // words of all rows
  std::vector<int4> rinfo;      // [nrows] {c0, c1 (-1: none), r1, position of word 0}
  std::vector<int4> rinfo2;     // [nrows] {c2, c3 (-1: none), r2, r3}
  std::vector<long long> roff;  // [nrows] first word of the row
  std::vector<int> rwords;      // [nrows] words of the row
  std::vector<int> rtile;       // [nrows] words per time tile: 1024 (one run) or its tiles' window
  std::vector<int> prow;        // [npair + 1] first row of each group
  std::vector<int2> prange;     // [npair][kPairGMax - 1] {smallest, largest r_i}, i = 1..
  std::vector<int> row_of;      // [dm_count][npair] row of each trial and group
  std::vector<int4> rec;        // stage records, pair_rec_int4(cc) int4 each
  std::vector<int> tile_st;     // [ntiles + 1] first record of each tile
};
// Group tables for trials [dm_first, dm_first + dm_count) over the active
// channels, g channels a group (2 or 4), cc groups per stage (4 or 8), for
// ntt time tiles of output.
PairTables dedisp_pair_tables(const int *delays_host, int nchan, const int *chans_host, int nact,
                              int dm_first, int dm_count, int cc, int ntt, int g);
// Per group, the end of the rows that the tables' first `count` trials use
// (a beam whose DM ceiling cuts the list builds those rows only).
void pair_row_ends(const PairTables &t, int count, int *ends);
// Builds the rows, then sums them (two launches); `a` is a launch with mode
// 5 or 6 and dpt 16 over one beam, `one`, or over beams[0 .. nbeam) read on
// the device (the batched context, whose ring positions the device
// advances; up to kPairMaxBeams beams, their rows pair_rows_stride words
// apart, their items one after another from beams[0].item0, beam z's row
// ends at pair_rend + z * npair).
cudaError_t dedisperse_pairs(const DedispArgs &a, cudaStream_t s);
// Largest delay spread over the active channels of any dpt-trial tile.
int dedisp_spread(const int *delays_host, int nchan, const int *chans_host, int nact,
                  int dm_first, int dm_count, int dpt);

// ------------------------------------------------------- smoothing
// One beam of a smoothing / peak-finding launch (device array).
struct SmoothBeam {
  const float *dd;          // [ndms][dd_stride] dedispersed plane
  long dd_stride;
  float *boxes;             // [nw][h][ntime_out]: the launch's widths w0.. (pre-normalise)
  float *rowmean, *rowmax, *rowvar;  // [nbox][h]
  float *stats;             // [nbox][4] mean, std, -mean, 1/std
  float *gate;              // [4] mean0n, sigma0n, threshold, pass
  int *counts, *offsets;    // [nbox][h]
  int4 *cand_i;             // [cap] beam, dm_idx, width, samp
  float *cand_v;            // [cap] normalised value
  int *total;               // [1] candidates written so far (capped at cap)
  const int *active;        // searched this gulp (0: every kernel skips the beam)
  int h;                    // rows: ndms - 2
  int row0;                 // first global row of the beam
  int cap;                  // candidate cap of the beam
  int beam_id;              // reported beam index
};

struct SmoothArgs {
  const SmoothBeam *beams;  // device [nbeam]
  int nbeam;
  const int *row_beam;      // device [nrows]: beam of each global row
  int nrows;                // sum of the beams' h
  int ntime_dd, ntime_out;
  int nbox, wmin, wmax, anchor;
  int w0, nw;               // widths of this launch: w0 .. w0 + nw - 1
  const float *taps;        // middle-row taps of every width, padded
  const int *tap_off;       // [nbox] offset into taps
  const int *tap_n;         // [nbox] padded tap count (multiple of 16)
  float snr;
  int split;                // FIR: first width of the second width group
                            // (w0 + nw: one group); set by smooth_planes
  int nogate;               // peaks whatever sigma0 (DEBUG_ALWAYS_FIND_PEAKS)
};
// Shared memory of the FIR launch.
size_t fir_smem_bytes(const SmoothArgs &a);
cudaError_t smooth_planes(const SmoothArgs &a, cudaStream_t s);
// scale = 1: per-width mean/std (normalisation); 0: planes left as they
// are.  A launch holding width 0 then forms the beams' gate statistics.
cudaError_t smooth_stats(const SmoothArgs &a, cudaStream_t s, int scale);
// Candidates of the launch's widths, appended to each beam's list after
// those of earlier widths (reset `total` before width 0).
cudaError_t find_peaks(const SmoothArgs &a, cudaStream_t s);
// Normalised copy of beam 0's planes (inspection).
cudaError_t normalise_copy(const SmoothArgs &a, float *dst, cudaStream_t s);

// ----------------------------------------------------- ring position
// Ring positions of the gulp being processed, kept in device memory so that
// a captured CUDA graph can be replayed gulp after gulp.
struct GulpPos {
  long win0;                // window start of a full-ring (R-sample) window
  long wpos;                // where the gulp is written: (win0 + R - gulp) % R
  int gulp_index;           // gulps processed before this one
  int pad;
};

}  // namespace hg
