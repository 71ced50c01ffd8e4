// hg_plan.h -- host plan math shared by the hdd_ API and the search context.
#pragma once

#include "hella_dedisp.h"
#include "hg_internal.h"

#include <vector>

namespace hg {

std::vector<float> generate_dm_list(double dm_start, double dm_end, double ti_us, double tol,
                                    int nchan, double dt_s, double f0, double df);
std::vector<float> delay_table(int nchan, double dt_s, double f0, double df);
std::vector<int> dm_delays(const std::vector<float> &dms, const std::vector<float> &table);

// Dedispersion tile tables for trials [first, first + count) with dpt
// trials per tile (0: the largest that fits cc-channel stages): host copy
// (cached per range and shape) and device copy (uploaded on first use).
const DedispTables &plan_host_tables(hdd_plan p, int first, int count, int dpt = 0, int cc = 8);
struct DeviceTables {
  const int4 *meta;
  const int *off;
  int dpt, max_spread, nact, cc;
};
hdd_error plan_device_tables(hdd_plan p, int first, int count, DeviceTables *out, int dpt = 0,
                             int cc = 8);
// Add-mode-4 tables for trials [first, first + count) over the plan's
// active channels: host copy cached per range, device copy uploaded on first use.
struct SubDeviceTables {
  const int4 *meta;
  const int2 *index;
  const int *pool;
  int max_spread, max_words, max_rec, nact;
};
hdd_error plan_sub_tables(hdd_plan p, int first, int count, SubDeviceTables *out);
// Points a launch at add-mode-4 tables (16-trial tiles; items must be counted
// for that tile size).
void use_sub_tables(DedispArgs *a, const SubDeviceTables &t);
// Add-mode-5/6 tables (rows of g = 2 or 4 channels) for trials [first,
// first + count) over the plan's active channels with cc groups per stage
// and ntt time tiles: host copy cached per range and shape, device copy and
// row buffer set up on first use.
struct PairDeviceTables {
  const int4 *rinfo;
  const int4 *rinfo2;
  const long long *roff;
  const int *rwords;
  const int *rtile;
  const int *prow;
  const int2 *prange;
  const int4 *rec;
  const int *tile_st;
  uint32_t *rows;
  int npair, span, stage, nact, cc, g;
  long npos, words;  // positions the rows cover; words of one beam's rows
};
// rows = false: the tables only (the caller holds the rows; `rows` is null).
hdd_error plan_pair_tables(hdd_plan p, int first, int count, int cc, int ntt, int g, PairDeviceTables *out,
                           bool rows = true);
// Builds (or keeps) the plan's host group-row tables for that range and shape.
hdd_error pair_host_tables(hdd_plan p, int first, int count, int cc, int ntt, int g);
// Frees the add-mode-5 device tables and rows (set up again on next use).
void plan_pair_release(hdd_plan p);
// Device bytes those tables and their rows take (builds the host copy).
hdd_error plan_pair_bytes(hdd_plan p, int first, int count, int cc, int ntt, int g, size_t *bytes);
// Per pair, the end of the rows that the first `count` trials use, for the
// tables last set up from trial 0 (a beam whose DM ceiling cuts the list).
hdd_error plan_pair_row_ends(hdd_plan p, int count, int *ends);
// Points a single-beam launch at add-mode-5 tables (16-trial tiles; items
// must be counted for that tile size).
void use_pair_tables(DedispArgs *a, const PairDeviceTables &t);
// Launch arguments for one beam over a plan's device tables.
DedispArgs single_beam_args(const DeviceTables &tb, const uint32_t *packed, long R, long win0,
                            int dm_first, int dm_count, int nout, float *out, long out_stride,
                            int *err);

// Read-only view of a plan's host tables.
struct PlanView {
  int device;
  void *stream;
  int nchans, ndms, max_delay, nact;
  const int *delays;  // [ndms][nchans]
  const int *chans;   // [nact] active channels
};
PlanView plan_view(hdd_plan p);

}  // namespace hg
