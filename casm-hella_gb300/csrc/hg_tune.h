// hg_tune.h -- dedispersion tile-shape search shared by the single-beam and
// batched search contexts.
#pragma once

#include "hella_search.h"

#include <cuda_runtime.h>

#include <functional>

namespace hg {

// Shapes the dedispersion kernels implement.
inline bool tuning_ok(const hella_tuning &t) {
  const bool dpt_ok = t.dm_per_block == 0 || t.dm_per_block == 1 || t.dm_per_block == 2 ||
                      t.dm_per_block == 4 || t.dm_per_block == 8 || t.dm_per_block == 16;
  return dpt_ok && (t.chan_chunk == 8 || t.chan_chunk == 16) &&
         (t.stages == 0 || (t.stages >= 2 && t.stages <= 4)) && t.group >= 1 && t.group <= 4096 &&
         t.add_mode >= 0 && t.add_mode <= 6 &&
         (t.add_mode < 4 || t.dm_per_block == 0 || t.dm_per_block == 16);
}

// Coordinate search from `start`: add mode, channel chunk, DM tile, pipeline
// depth and group, each varied with the others held at the best so far, two
// rounds.  time_shape(t, &ms) times one shape; HELLA_ERR_INVALID_ARG (a
// shape the DM list cannot use), HELLA_ERR_CUDA (a launch the device
// refused, e.g. staging beyond shared memory), HELLA_ERR_ALLOC and
// HELLA_ERR_BUDGET (add mode 5's or 6's rows beyond the free memory or the
// HBM budget) skip the shape, any other error ends the search.
inline hella_status tune_shapes(const hella_tuning &start,
                                const std::function<hella_status(const hella_tuning &, float *)> &time_shape,
                                hella_tuning *best_out, float *best_ms_out) {
  hella_tuning best = start;
  float best_ms = 3.4e38f;
  hella_status s = time_shape(best, &best_ms);
  if (s == HELLA_ERR_INVALID_ARG || s == HELLA_ERR_CUDA || s == HELLA_ERR_ALLOC || s == HELLA_ERR_BUDGET) {
    cudaGetLastError();  // a start shape this context cannot run: start from one every DM list runs
    best.dm_per_block = 0;
    best.chan_chunk = 8;
    best.stages = 0;
    best.add_mode = 0;
    s = time_shape(best, &best_ms);
  }
  if (s != HELLA_OK) return s;
  auto try_shape = [&](hella_tuning t) -> hella_status {
    if (!tuning_ok(t)) return HELLA_OK;
    float ms = 0.f;
    const hella_status r = time_shape(t, &ms);
    if (r == HELLA_ERR_INVALID_ARG || r == HELLA_ERR_CUDA || r == HELLA_ERR_ALLOC || r == HELLA_ERR_BUDGET) {
      cudaGetLastError();
      return HELLA_OK;
    }
    if (r != HELLA_OK) return r;
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
    return HELLA_OK;
  };
  for (int round = 0; round < 2; ++round) {
    for (int m : {0, 1, 2, 3, 5, 6}) {  // add mode 4 measured slower on every workload: not searched
      hella_tuning t = best;
      t.add_mode = m;
      if ((s = try_shape(t)) != HELLA_OK) return s;
    }
    for (int cc : {8, 16}) {
      hella_tuning t = best;
      t.chan_chunk = cc;
      if ((s = try_shape(t)) != HELLA_OK) return s;
    }
    for (int d : {16, 8}) {
      hella_tuning t = best;
      t.dm_per_block = d;
      if ((s = try_shape(t)) != HELLA_OK) return s;
    }
    for (int nb : {2, 3, 4}) {
      hella_tuning t = best;
      t.stages = nb;
      if ((s = try_shape(t)) != HELLA_OK) return s;
    }
    for (int g : {2, 4, 8, 16, 32}) {
      hella_tuning t = best;
      t.group = g;
      if ((s = try_shape(t)) != HELLA_OK) return s;
    }
  }
  *best_out = best;
  *best_ms_out = best_ms;
  return HELLA_OK;
}

// Best of `reps` timed runs of `run` on `stream` (one untimed run first),
// milliseconds.
inline hella_status time_runs(cudaStream_t stream, int reps, const std::function<hella_status()> &run,
                              float *ms) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  float best = 3.4e38f;
  hella_status s = HELLA_OK;
  for (int r = 0; r <= reps && s == HELLA_OK; ++r) {
    if (cudaEventRecord(e0, stream) != cudaSuccess) {
      s = HELLA_ERR_CUDA;
      break;
    }
    if ((s = run()) != HELLA_OK) break;
    if (cudaEventRecord(e1, stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
      s = HELLA_ERR_CUDA;
      break;
    }
    float m = 0.f;
    cudaEventElapsedTime(&m, e0, e1);
    if (r > 0 && m < best) best = m;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != HELLA_OK) {
    cudaGetLastError();
    return s;
  }
  *ms = best;
  return HELLA_OK;
}

}  // namespace hg
