// flagger.cu -- casm-hella's spectral RFI flagger and normaliser on GB300.
//
// Reference: src/hella/src/flagger.cu:345-411 (fast_flagger) with the
// default configuration (no SCRUNCH lines): bandpass_flag (:216-242), then
// apply_scrunch(8, 8, 100, flag=0, ts=1) (:385-401), then transpose_output
// (transpose.cu:48-76).
//
// Design.  The reference materialises an fp16 copy of the gulp and rewrites
// it ~14 times.  Here the fp16 plane is never stored: up to the time-series
// correction every value depends only on its channel and its u8 input level,
// so each stage publishes a 256-entry lookup table per channel and every
// reduction pass re-reads the u8 gulp (1 byte per sample) and maps it
// through the table.  The per-time division and the final normalisation are
// applied on the fly.  Each reduction reproduces the reference's order:
//   calc_bandpass_new  (flagger.cu:86-112)   32 lane partials in time order,
//                                            warp shuffle tree, / width
//   computeRowMeans    (normalization.cu:19-69) 256 strided partials, warp
//   computeRowVariances(normalization.cu:72-122) trees, 8-warp sum, / width
//   calculate_stddev host loops (normalization.cu:138-153) sequential over
//                                            channels, done by one thread
//   measure_ts         (timeseries.cu:19-36)  fp16 running sum over channels
// so the output bytes equal the reference's on the same gulp.
#include "hg_internal.h"
#include "hella_search.h"

#include <algorithm>
#include <cmath>

namespace hg {
namespace {


__device__ __forceinline__ __half hzero() { return __float2half_rn(0.f); }
__device__ __forceinline__ __half hone() { return __float2half_rn(1.f); }

// Value of u8 level v of (beam b, channel c) after flagger stage `stage`:
//  1 bandpass_correct   divide_by_bp (flagger.cu:180-194)
//  2 normalize_data     (x + half(-mean)) * half(1/std) (flagger.cu:198-214)
//  3 spectral flag      1, or x + 1 (replace_data_and_add_bandpass :146-158)
//  4 bandpass_correct   of the final scrunch
__device__ __half chain_value(int stage, int v, const FlagState &st, int b,
                              int c) {
  const int bc = b * st.nchan + c;
  __half x = __float2half_rn((float)v);
  if (stage >= 1) {
    float bp = st.bp1[bc];
    x = bp > 0.f ? __hdiv(x, __float2half_rn(bp)) : hzero();
  }
  if (stage >= 2) x = __hmul(__hadd(x, st.hsc[b * 8 + 0]), st.hsc[b * 8 + 1]);
  if (stage >= 3) x = st.flag2[bc] ? hone() : __hadd(x, hone());
  if (stage >= 4) {
    float bp = st.bp3[bc];
    x = bp > 0.f ? __hdiv(x, __float2half_rn(bp)) : hzero();
  }
  return x;
}

__global__ void k_build_lut(FlagState st, int stage) {
  const int c = blockIdx.x, b = blockIdx.y, v = threadIdx.x;
  st.lut[((size_t)b * st.nchan + c) * 256 + v] = chain_value(stage, v, st, b, c);
}

// The row-statistics pass in a four-channel form: lane t of a warp holds
// channels c0 + 4t .. c0 + 4t + 3 (one 32-bit load per row feeds four
// chains, each summed in the reference's order), warps hold columns.  The
// block's 128-channel slice of the table is staged as
// lut_s[level * kQC + channel] through 16-byte loads of eight levels.
constexpr int kQC = 128;
constexpr int kRowT = 512;  // threads per block
constexpr size_t kLutSlice = (size_t)256 * kQC * sizeof(__half);

// Stages the table slice of channels c0 .. c0 + NC - 1 of beam b as
// lut_s[level * NC + channel] (channels past nchan are left alone): each
// thread loads eight levels of one channel with a 16-byte load, and the
// lanes of a warp, holding consecutive channels, store without conflicts.
template <int NC>
__device__ __forceinline__ void load_lut_slice(__half *lut_s, const __half *lut, int nchan, int b, int c0) {
  const int ncl = min(NC, nchan - c0);
  const __half *lb = lut + ((size_t)b * nchan + c0) * 256;
  for (int i = threadIdx.x; i < NC * 32; i += blockDim.x) {
    const int cc = i % NC, vb = i / NC;  // levels 8vb .. 8vb+7 of channel cc
    if (cc < ncl) {
      const uint4 q = *reinterpret_cast<const uint4 *>(lb + (size_t)cc * 256 + 8 * vb);
      const __half *h = reinterpret_cast<const __half *>(&q);
#pragma unroll
      for (int k = 0; k < 8; ++k) lut_s[(8 * vb + k) * NC + cc] = h[k];
    }
  }
}

// calc_bandpass_new partials: lane l of channel c sums samples l, l+32, ...
// (below 32*floor(w/32)) in time order.  Block = 32 channels x 8 lanes, one
// chain a thread (65536 chains for 2048 channels: too few for the
// four-channel form to hide the memory latency); the row bytes are loaded
// kLaneB at a time so that as many loads are in flight (64 a thread, about
// 4 MB over the GPU; the two-blocks bound lets the compiler give them the
// registers, 96, where it would otherwise fit 32 and interleave them with
// the sums).  The table slice is staged as lut_s[level][channel] through
// 16-byte loads of eight levels.
constexpr int kLaneC = 32, kLaneB = 64;
__global__ void __launch_bounds__(256, 2) k_lane_partials(const uint8_t *__restrict__ gulp,
                                                       const __half *__restrict__ lut,
                                                       float *__restrict__ part, int nchan, int w) {
  __shared__ __half lut_s[256][kLaneC];
  const int b = blockIdx.z, c0 = blockIdx.x * kLaneC;
  load_lut_slice<kLaneC>(&lut_s[0][0], lut, nchan, b, c0);
  __syncthreads();
  const int cl = threadIdx.x & 31, l = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int c = c0 + cl;
  const uint8_t *g = gulp + (size_t)b * w * nchan + (size_t)l * nchan + c;
  const size_t step = (size_t)32 * nchan;
  const int np = w / 32;
  float s = 0.f;
  int i = 0;
  for (; i + kLaneB <= np; i += kLaneB) {
    uint32_t v[kLaneB];
#pragma unroll
    for (int u = 0; u < kLaneB; ++u) v[u] = g[(size_t)(i + u) * step];
#pragma unroll
    for (int u = 0; u < kLaneB; ++u) s = __fadd_rn(s, __half2float(lut_s[v[u]][cl]));
  }
  for (; i < np; ++i) s = __fadd_rn(s, __half2float(lut_s[g[(size_t)i * step]][cl]));
  part[((size_t)b * nchan + c) * 32 + l] = s;
}

// computeRowMeans / computeRowVariances partials: column j of channel c
// sums columns j, j+256, ... below nw = 256*floor(w/256).  TS: values
// divided by half(ts[t]) (divide_by_ts, timeseries.cu:38-55).  VAR:
// (x - mean)^2 with the fused multiply-add the reference's compiler emits.
// The two-blocks bound gives the unrolled loads registers (44-64 instead of
// 32), as in k_lane_partials.
template <bool VAR, bool TS>
__global__ void __launch_bounds__(kRowT, 2) k_row_partials(const uint8_t *__restrict__ gulp, FlagState st,
                                                            int which) {
  extern __shared__ __align__(16) __half lut4_s[];
  const int b = blockIdx.z, c0 = blockIdx.x * kQC, nchan = st.nchan, w = st.gulp;
  load_lut_slice<kQC>(lut4_s, st.lut, nchan, b, c0);
  __syncthreads();
  const int cq = 4 * (threadIdx.x & 31), c = c0 + cq;
  const int j = blockIdx.y * (kRowT / 32) + (threadIdx.x >> 5);
  if (c >= nchan) return;
  const uint8_t *g = gulp + (size_t)b * w * nchan + (size_t)j * nchan + c;
  const __half *hts = st.hts + (size_t)b * w + j;
  const size_t step = (size_t)256 * nchan;
  const int nk = w / 256;
  const float mean = VAR ? st.scal[b * 8 + 2 * which] : 0.f;
  const __half *ls = lut4_s + cq;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
  for (int k = 0; k < nk; ++k) {
    const uint32_t x = *reinterpret_cast<const uint32_t *>(g + k * step);
    __half th;
    if (TS) th = hts[k * 256];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      __half hv = ls[((x >> (8 * q)) & 255u) * kQC + q];
      if (TS) hv = __hdiv(hv, th);
      const float f = __half2float(hv);
      if (VAR) {
        const float d = __fsub_rn(f, mean);
        acc[q] = __fmaf_rn(d, d, acc[q]);
      } else {
        acc[q] = __fadd_rn(acc[q], f);
      }
    }
  }
  float *pp = st.part + ((size_t)b * nchan + c) * 256 + j;
#pragma unroll
  for (int q = 0; q < 4; ++q) pp[q * 256] = acc[q];
}

// Warp tree over the 32 lane partials, / w (flagger.cu:103-111).  One warp
// per (beam, channel).  mode 0: bp1, 1: bp2 + spectral flag, 2: bp3.
__global__ void k_lane_finish(FlagState st, int mode) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= st.nbeam * st.nchan) return;
  float v = st.part[(size_t)gw * 32 + lane];
  for (int off = 16; off > 0; off /= 2) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
  if (lane == 0) {
    float bp = __fdiv_rn(v, (float)st.gulp);
    if (mode == 0) st.bp1[gw] = bp;
    if (mode == 1) {
      st.bp2[gw] = bp;
      st.flag2[gw] = (bp < st.spec_min || bp > st.spec_max) ? 1 : 0;
    }
    if (mode == 2) st.bp3[gw] = bp;
    if (mode == 3) st.bpx[gw] = bp;
  }
}

// Thread 0 of the reference's 256-thread block: each warp's shuffle tree,
// then warp totals 1..7 added in order, / nw.  One warp per channel.
__global__ void k_row_finish(FlagState st) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= st.nbeam * st.nchan) return;
  const float *p = st.part + (size_t)gw * 256;
  float tot = 0.f;
  for (int wi = 0; wi < 8; ++wi) {
    float v = p[wi * 32 + lane];
    for (int off = 16; off > 0; off /= 2) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
    tot = wi == 0 ? v : __fadd_rn(tot, v);
  }
  if (lane == 0) st.rowval[gw] = __fdiv_rn(tot, (float)(256 * (st.gulp / 256)));
}

// calculate_stddev's host loops (normalization.cu:138-153): sequential sum
// over channels, / nchan; the variance pass also forms the half-precision
// normalisation constants of normalize_data (flagger.cu:205-206).  Block =
// beam: the row values are staged in shared memory with coalesced loads,
// thread 0 adds them in channel order.
constexpr int kBeamT = 256, kMaxChan = 8192;  // the largest nchan accepted
template <bool VAR>
__global__ void __launch_bounds__(kBeamT) k_beam_sum(FlagState st, int which) {
  __shared__ float rv_s[kMaxChan];
  const int b = blockIdx.x;
  const float *rv = st.rowval + (size_t)b * st.nchan;
  for (int c = threadIdx.x; c < st.nchan; c += kBeamT) rv_s[c] = rv[c];
  __syncthreads();
  if (threadIdx.x != 0) return;
  float s = 0.f;
  for (int c = 0; c < st.nchan; ++c) s = __fadd_rn(s, rv_s[c]);
  s = __fdiv_rn(s, (float)st.nchan);
  if (!VAR) {
    st.scal[b * 8 + 2 * which] = s;
  } else {
    float sd = __fsqrt_rn(s);
    float mean = st.scal[b * 8 + 2 * which];
    st.scal[b * 8 + 2 * which + 1] = sd;
    st.hsc[b * 8 + 2 * which] = __float2half_rn(-mean);
    st.hsc[b * 8 + 2 * which + 1] = __float2half_rn(__fdiv_rn(1.f, sd));
  }
}

// med_filter_bandpass (median_filter.cpp:85-107, median_filter :36-77) with
// a window of win (odd) channels: channel i in [h, nchan - h) takes the
// middle element of its sorted window (h = win / 2), the first h channels
// take channel h's value and the last h channel nchan - h - 1's.  Any sort
// leaves the same middle element, so the values are the reference's.  One
// block per beam, in place: the row is staged in shared memory first.
__global__ void __launch_bounds__(kBeamT) k_bp_median(float *__restrict__ bp, int nchan, int win) {
  __shared__ float row[kMaxChan];
  float *r = bp + (size_t)blockIdx.x * nchan;
  for (int c = threadIdx.x; c < nchan; c += blockDim.x) row[c] = r[c];
  __syncthreads();
  const int h = win / 2;
  for (int c = threadIdx.x; c < nchan; c += blockDim.x) {
    const int i = min(max(c, h), nchan - h - 1);
    float w[kMaxBpMedian];
    for (int k = 0; k < win; ++k) {  // insertion sort of the window
      const float v = row[i - h + k];
      int j = k - 1;
      while (j >= 0 && w[j] > v) {
        w[j + 1] = w[j];
        --j;
      }
      w[j + 1] = v;
    }
    r[c] = w[h];
  }
}

// k_lane_finish for mode, then the bandpass median filter where the
// reference's bandpass_correct applies it (modes 0, 2 and 3: every bandpass
// that data are divided by; not the spectral-flag bandpass of mode 1).
unsigned lane_finish(const FlagState &st, int mode, int fin_blocks, cudaStream_t s) {
  k_lane_finish<<<fin_blocks, 256, 0, s>>>(st, mode);
  if (mode == 1 || st.bp_median <= 1) return 1;
  float *bp = mode == 0 ? st.bp1 : mode == 2 ? st.bp3 : st.bpx;
  k_bp_median<<<st.nbeam, kBeamT, 0, s>>>(bp, st.nchan, st.bp_median);
  return 2;
}

// measure_ts: per sample, fp16 running sum over channels in channel order,
// then ts = float(sum) / nchan.  Block = 128 consecutive samples; rows and
// table slices are staged through shared memory 64 channels at a time.
// The gulp rows and table slices are staged with 4- and 16-byte loads
// (nchan % 32 == 0 keeps every 64-channel chunk whole and aligned).
constexpr int kTsT = 128, kTsC = 64;
__global__ void __launch_bounds__(kTsT) k_ts(const uint8_t *__restrict__ gulp,
                                             FlagState st) {
  __shared__ __align__(16) uint8_t rows_s[kTsT][kTsC + 4];
  __shared__ __align__(16) __half lut_s[kTsC][256];
  const int b = blockIdx.y, t0 = blockIdx.x * kTsT, nchan = st.nchan, w = st.gulp;
  const int tid = threadIdx.x;
  const uint8_t *g = gulp + (size_t)b * w * nchan + (size_t)t0 * nchan;
  const __half *lb = st.lut + (size_t)b * nchan * 256;
  __half s = hzero();
  for (int c0 = 0; c0 < nchan; c0 += kTsC) {
    const int nc = min(kTsC, nchan - c0);
    __syncthreads();
    for (int i = tid; i < kTsT * (kTsC / 4); i += kTsT) {
      const int r = i / (kTsC / 4), c4 = 4 * (i % (kTsC / 4));
      if (c4 < nc && t0 + r < w)
        *reinterpret_cast<uint32_t *>(&rows_s[r][c4]) =
            *reinterpret_cast<const uint32_t *>(g + (size_t)r * nchan + c0 + c4);
    }
    const uint4 *lsrc = reinterpret_cast<const uint4 *>(lb + (size_t)c0 * 256);
    uint4 *ldst = reinterpret_cast<uint4 *>(&lut_s[0][0]);
    for (int i = tid; i < nc * 256 / 8; i += kTsT) ldst[i] = lsrc[i];
    __syncthreads();
    if (t0 + tid < w)
      for (int cc = 0; cc < nc; ++cc) s = __hadd(s, lut_s[cc][rows_s[tid][cc]]);
  }
  if (t0 + tid < w) {
    float ts = __fdiv_rn(__half2float(s), (float)nchan);
    st.ts[(size_t)b * w + t0 + tid] = ts;
    st.hts[(size_t)b * w + t0 + tid] = __float2half_rn(ts);
  }
}

// transpose_output (transpose.cu:321-331): u8 = trunc(clamp(255/14 (x+4))).
__device__ __forceinline__ uint8_t requant(__half h) {
  float v = __half2float(h);
  const float scf = 255.f / 14.f;
  v = __fmul_rn(scf, __fadd_rn(v, 4.f));
  if (v < 0.f) v = 0.f;
  if (v > 255.f) v = 255.f;
  return (uint8_t)v;
}

// Final stage: divide_by_ts, normalize_data, requantise, and write the
// channel-major ring.  Block = 32 channels x kOutT samples: the channels'
// table slice is staged in shared memory (as in k_lane_partials), each
// thread maps samples of one channel into a channel-major byte tile
// (row stride kOutT + 4: conflict-free both ways), and the tile leaves as
// 4-byte words, 128 bytes of one channel per warp.  The ring position of a
// gulp (and R) are multiples of 32, so no word straddles the ring's end.
constexpr int kOutT = 512, kOutC = 32;
__global__ void __launch_bounds__(256) k_flag_out(const uint8_t *__restrict__ gulp, FlagState st,
                                                  uint8_t *__restrict__ plain, long R, long wpos,
                                                  const GulpPos *dpos) {
  if (dpos) wpos = dpos->wpos;
  __shared__ __half lut_s[256][kOutC];
  __shared__ __align__(16) uint8_t tile[kOutC][kOutT + 4];
  const int b = blockIdx.z, c0 = blockIdx.x * kOutC, t0 = blockIdx.y * kOutT;
  const int nchan = st.nchan, w = st.gulp, tid = threadIdx.x;
  load_lut_slice<kOutC>(&lut_s[0][0], st.lut, nchan, b, c0);
  __syncthreads();
  const __half a2 = st.hsc[b * 8 + 2], m2 = st.hsc[b * 8 + 3];
  const uint8_t *g = gulp + (size_t)b * w * nchan + c0;
  const __half *hts = st.hts + (size_t)b * w;
  const int cl = tid & 31, tr = tid >> 5;
  const int nt = min(kOutT, w - t0);
#pragma unroll 4
  for (int tt = tr; tt < nt; tt += 8) {
    const int t = t0 + tt;
    __half x = __hdiv(lut_s[g[(size_t)t * nchan + cl]][cl], hts[t]);
    x = __hmul(__hadd(x, a2), m2);
    tile[cl][tt] = requant(x);
  }
  __syncthreads();
  uint8_t *pb = plain + ((size_t)b * nchan + c0) * R;
  const int nq = nt / 4;  // w % 32 == 0
  for (int i = tid; i < kOutC * nq; i += 256) {
    const int c = i / nq, q = i - c * nq;
    long pos = wpos + t0 + 4 * q;
    if (pos >= R) pos -= R;
    *reinterpret_cast<uint32_t *>(pb + (size_t)c * R + pos) = *reinterpret_cast<const uint32_t *>(&tile[c][4 * q]);
  }
}

}  // namespace

namespace {
// ------------------------------------------------ SCRUNCH entries (planes)
// Kernels of the plane path, each the counterpart of a reference kernel run
// on the fp16 copy of the gulp; index `i` runs over [nbeam][nchan][gulp].

// The data after bandpass_flag (table stage 3) as a channel-major plane.
__global__ void k_plane_init(const uint8_t *__restrict__ gulp, FlagState st) {
  __shared__ uint8_t tile[32][33];
  const int b = blockIdx.z, c0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y, nchan = st.nchan, w = st.gulp;
  const uint8_t *g = gulp + (size_t)b * w * nchan;
#pragma unroll
  for (int j = 0; j < 32; j += 8) tile[ty + j][tx] = g[(size_t)(t0 + ty + j) * nchan + c0 + tx];
  __syncthreads();
  const __half *lb = st.lut + (size_t)b * nchan * 256;
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int c = c0 + ty + j;
    st.P[((size_t)b * nchan + c) * w + t0 + tx] = lb[(size_t)c * 256 + tile[tx][ty + j]];
  }
}

// calc_bandpass_new partials of the plane (lane l: samples l, l+32, ...).
// One warp per (beam, channel).
__global__ void k_plane_lanes(FlagState st) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (gw >= st.nbeam * st.nchan) return;
  const __half *p = st.P + (size_t)gw * st.gulp + lane;
  const int np = st.gulp / 32;
  float s = 0.f;
  for (int i = 0; i < np; ++i) s = __fadd_rn(s, __half2float(p[(size_t)i * 32]));
  st.part[(size_t)gw * 32 + lane] = s;
}

// divide_by_bp (flagger.cu:180-194) with bandpass bp [nbeam][nchan].
__global__ void k_plane_div(FlagState st, const float *bp) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float v = bp[i / st.gulp];
    st.P[i] = v > 0.f ? __hdiv(st.P[i], __float2half_rn(v)) : hzero();
  }
}

// computeRowMeans / computeRowVariances partials of the plane.
template <bool VAR>
__global__ void __launch_bounds__(256) k_plane_rows(FlagState st, int which) {
  const int c = blockIdx.x, b = blockIdx.y, j = threadIdx.x, w = st.gulp;
  const __half *p = st.P + ((size_t)b * st.nchan + c) * w + j;
  const float mean = VAR ? st.scal[b * 8 + 2 * which] : 0.f;
  float s = 0.f;
  for (int k = 0; k < w / 256; ++k) {
    const float f = __half2float(p[(size_t)k * 256]);
    if (VAR) {
      const float d = __fsub_rn(f, mean);
      s = __fmaf_rn(d, d, s);
    } else {
      s = __fadd_rn(s, f);
    }
  }
  st.part[((size_t)b * st.nchan + c) * 256 + j] = s;
}

// normalize_data (flagger.cu:198-214) with the constants of slot `which`.
__global__ void k_plane_norm(FlagState st, int which) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp, per = (size_t)st.nchan * st.gulp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / per);
    st.P[i] = __hmul(__hadd(st.P[i], st.hsc[b * 8 + 2 * which]), st.hsc[b * 8 + 2 * which + 1]);
  }
}

// npp_convolve_handler (convolution.cu:20-55): an xw (time) x yw (channel)
// box of equal taps k, anchor (xw/2, yw/2), replicate border, fp32 sum of
// fp16 input, fp16 output.  Tap (j, i) multiplies input (c + ay - j,
// t + ax - i); the sum runs j outer, i inner, one fmaf per tap.  A block
// computes 64 samples x 16 channels from a staged halo tile.
constexpr int kBoxT = 64, kBoxC = 16;
__global__ void __launch_bounds__(256) k_box(const __half *__restrict__ in, __half *__restrict__ out,
                                             int nchan, int w, int xw, int yw, float k) {
  extern __shared__ float tile[];
  const int b = blockIdx.z, t0 = blockIdx.x * kBoxT, c0 = blockIdx.y * kBoxC, tid = threadIdx.x;
  const int ax = xw / 2, ay = yw / 2;
  const int tw = kBoxT + xw - 1, th = kBoxC + yw - 1;
  const int cb = c0 + ay - (yw - 1), tb = t0 + ax - (xw - 1);  // tile origin (before clamping)
  const __half *src = in + (size_t)b * nchan * w;
  for (int q = tid; q < tw * th; q += 256) {
    const int r = q / tw, col = q - r * tw;
    const int cc = min(max(cb + r, 0), nchan - 1), tt = min(max(tb + col, 0), w - 1);
    tile[q] = __half2float(src[(size_t)cc * w + tt]);
  }
  __syncthreads();
  const int tl = tid & (kBoxT - 1);
  for (int cl = tid >> 6; cl < kBoxC; cl += 256 / kBoxT) {
    const int c = c0 + cl, t = t0 + tl;
    float acc = 0.f;
    for (int j = 0; j < yw; ++j) {
      const float *row = tile + (size_t)(cl + yw - 1 - j) * tw + tl + xw - 1;
      for (int i = 0; i < xw; ++i) acc = __fmaf_rn(k, row[-i], acc);
    }
    if (c < nchan && t < w) out[((size_t)b * nchan + c) * w + t] = __float2half_rn(acc);
  }
}

// threshold_data (flagger.cu:162-176): mask 1 where the smoothed value
// exceeds +-half(thr).
__global__ void k_plane_thresh(FlagState st, __half hp, __half hn) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp;
  const float p = __half2float(hp), m = __half2float(hn);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float v = __half2float(st.S[i]);
    st.M[i] = (v > p || v < m) ? hone() : hzero();
  }
}

// replace_data (flagger.cu:128-144) with FLAG1/FLAG2, then add_number 1.
__global__ void k_plane_replace(FlagState st) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)((i / st.gulp) % st.nchan);
    __half v = st.P[i];
    if (__half2float(st.S[i]) > 0.f) v = hzero();
    if (c >= st.flag_lo && c < st.flag_hi) v = hzero();
    st.P[i] = __hadd(v, hone());
  }
}

// calc_bandpass (flagger.cu:50-81) of the grown mask: thread t sums its
// contiguous floor(w/256) samples in fp16, / half(256 floor(w/256)), then an
// fp16 tree.  Block = (channel, beam).
__global__ void __launch_bounds__(256) k_plane_bp16(FlagState st) {
  __shared__ __half ps[256];
  const int c = blockIdx.x, b = blockIdx.y, t = threadIdx.x, np = st.gulp / 256;
  const __half *p = st.S + ((size_t)b * st.nchan + c) * st.gulp + (size_t)t * np;
  __half s = hzero();
  for (int i = 0; i < np; ++i) s = __hadd(s, p[i]);
  ps[t] = __hdiv(s, __float2half_rn((float)(256 * np)));
  __syncthreads();
  for (int h = 128; h >= 1; h /= 2) {
    if (t < h) ps[t] = __hadd(ps[t], ps[t + h]);
    __syncthreads();
  }
  if (t == 0) st.fsb[(size_t)b * st.nchan + c] = __half2float(ps[0]);
}

// replace_data_and_add_bandpass (flagger.cu:146-158): flagged channels 1,
// the others x + 1.
__global__ void k_plane_spec(FlagState st) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    st.P[i] = st.flag2[i / st.gulp] ? hone() : __hadd(st.P[i], hone());
}

// add_bandpass into d_flagSpec (flagger.cu:333-334), beams in order.
__global__ void k_flagspec_add(FlagState st) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= st.nchan) return;
  float f = st.flagspec[c];
  for (int b = 0; b < st.nbeam; ++b) f = __fadd_rn(f, st.fsb[(size_t)b * st.nchan + c]);
  st.flagspec[c] = f;
}

// measure_ts + divide_by_ts (timeseries.cu:19-55) on the plane.
__global__ void k_plane_ts(FlagState st) {
  const int b = blockIdx.y, t = blockIdx.x * blockDim.x + threadIdx.x, w = st.gulp;
  if (t >= w) return;
  const __half *p = st.P + (size_t)b * st.nchan * w + t;
  __half s = hzero();
  for (int c = 0; c < st.nchan; ++c) s = __hadd(s, p[(size_t)c * w]);
  const float ts = __fdiv_rn(__half2float(s), (float)st.nchan);
  st.ts[(size_t)b * w + t] = ts;
  st.hts[(size_t)b * w + t] = __float2half_rn(ts);
}

__global__ void k_plane_tsdiv(FlagState st) {
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp, per = (size_t)st.nchan * st.gulp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / per, t = i % st.gulp;
    st.P[i] = __hdiv(st.P[i], st.hts[b * st.gulp + t]);
  }
}

// transpose_output of the plane into the channel-major ring.
__global__ void k_plane_out(FlagState st, uint8_t *__restrict__ plain, long R, long wpos, const GulpPos *dpos) {
  if (dpos) wpos = dpos->wpos;
  const int b = blockIdx.z, c = blockIdx.y, w = st.gulp;
  const __half *p = st.P + ((size_t)b * st.nchan + c) * w;
  uint8_t *row = plain + ((size_t)b * st.nchan + c) * R;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w; t += gridDim.x * blockDim.x) {
    long pos = wpos + t;
    if (pos >= R) pos -= R;
    row[pos] = requant(p[t]);
  }
}

}  // namespace

namespace {

// SCRUNCH entries and the final scrunch on fp16 planes (flagger.cu:365-401),
// from the data after bandpass_flag.
cudaError_t scrunch_planes(const FlagState &st, const void *gulp, uint8_t *plain, long R, long wpos,
                           const GulpPos *dpos, cudaStream_t s) {
  const dim3 lutg(st.nchan, st.nbeam);
  const int fin_blocks = (st.nbeam * st.nchan * 32 + 255) / 256;
  const size_t n = (size_t)st.nbeam * st.nchan * st.gulp;
  const int eb = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  const dim3 chg(st.nchan, st.nbeam);
  unsigned launches = 0;
  auto normalize = [&](int which) {
    k_plane_rows<false><<<chg, 256, 0, s>>>(st, which);
    k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
    k_beam_sum<false><<<st.nbeam, kBeamT, 0, s>>>(st, which);
    k_plane_rows<true><<<chg, 256, 0, s>>>(st, which);
    k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
    k_beam_sum<true><<<st.nbeam, kBeamT, 0, s>>>(st, which);
    k_plane_norm<<<eb, 256, 0, s>>>(st, which);
    launches += 7;
  };
  auto bandpass_correct = [&](int mode, const float *bp) {
    k_plane_lanes<<<fin_blocks, 256, 0, s>>>(st);
    launches += lane_finish(st, mode, fin_blocks, s);
    k_plane_div<<<eb, 256, 0, s>>>(st, bp);
    launches += 2;
  };
  if (st.f16_input) {
    // the DADA path (transpose.cu:87-90): the gulp is the fp16 plane; bandpass_flag on it
    cudaError_t e = cudaMemcpyAsync(st.P, gulp, n * sizeof(__half), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    bandpass_correct(0, st.bp1);
    normalize(0);
    k_plane_lanes<<<fin_blocks, 256, 0, s>>>(st);
    k_lane_finish<<<fin_blocks, 256, 0, s>>>(st, 1);
    k_plane_spec<<<eb, 256, 0, s>>>(st);
    launches += 3;
  } else {
    k_build_lut<<<lutg, 256, 0, s>>>(st, 3);
    k_plane_init<<<dim3(st.nchan / 32, st.gulp / 32, st.nbeam), dim3(32, 8), 0, s>>>(
        static_cast<const uint8_t *>(gulp), st);
    launches += 2;
  }
  for (int e = 0; e < st.nscrunch; ++e) {
    const int xw = st.sc_t[e], yw = st.sc_f[e];
    bandpass_correct(3, st.bpx);
    normalize(2);
    const float k = (float)(1. / xw / yw);
    const float thr = (float)(st.sc_thresh[e] / std::sqrt(1. * xw * yw));
    const __half hp = __float2half_rn(thr), hn = __float2half_rn((float)(-1. * thr));
    const dim3 bg((st.gulp + kBoxT - 1) / kBoxT, (st.nchan + kBoxC - 1) / kBoxC, st.nbeam);
    const size_t smem = sizeof(float) * (size_t)(kBoxT + xw - 1) * (kBoxC + yw - 1);
    k_box<<<bg, 256, smem, s>>>(st.P, st.S, st.nchan, st.gulp, xw, yw, k);
    k_plane_thresh<<<eb, 256, 0, s>>>(st, hp, hn);
    k_box<<<bg, 256, smem, s>>>(st.M, st.S, st.nchan, st.gulp, xw, yw, k);
    k_plane_replace<<<eb, 256, 0, s>>>(st);
    launches += 4;
    if (st.flagspec) {
      k_plane_bp16<<<chg, 256, 0, s>>>(st);
      k_flagspec_add<<<(st.nchan + 255) / 256, 256, 0, s>>>(st);
      launches += 2;
    }
  }
  // apply_scrunch(8, 8, 100, flag=0, ts=1)
  bandpass_correct(2, st.bp3);
  k_plane_ts<<<dim3((st.gulp + 127) / 128, st.nbeam), 128, 0, s>>>(st);
  k_plane_tsdiv<<<eb, 256, 0, s>>>(st);
  normalize(1);
  k_plane_out<<<dim3((st.gulp + 1023) / 1024, st.nchan, st.nbeam), 256, 0, s>>>(st, plain, R, wpos, dpos);
  launches += 3;
  count_launches(launches);
  return cudaGetLastError();
}

cudaError_t flag_impl(const FlagState &st, const void *gulp_in, uint8_t *plain, long R, long wpos,
                      const GulpPos *dpos, cudaStream_t s) {
  if (st.f16_input) return scrunch_planes(st, gulp_in, plain, R, wpos, dpos, s);
  const uint8_t *gulp = static_cast<const uint8_t *>(gulp_in);
  const dim3 lutg(st.nchan, st.nbeam);
  const dim3 laneg(st.nchan / kLaneC, 32 / 8, st.nbeam);
  const dim3 rowg((st.nchan + kQC - 1) / kQC, 256 / (kRowT / 32), st.nbeam);
  {  // the table slice is above the default 48 KB of dynamic shared memory
    const int lb = (int)kLutSlice;
    cudaError_t e = cudaFuncSetAttribute(k_row_partials<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_row_partials<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_row_partials<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_row_partials<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e != cudaSuccess) return e;
  }
  const int fin_blocks = (st.nbeam * st.nchan * 32 + 255) / 256;

  // bandpass_flag: bandpass_correct (calc_bandpass_new, divide_by_bp)
  k_build_lut<<<lutg, 256, 0, s>>>(st, 0);
  k_lane_partials<<<laneg, 256, 0, s>>>(gulp, st.lut, st.part, st.nchan, st.gulp);
  unsigned extra = lane_finish(st, 0, fin_blocks, s) - 1;
  k_build_lut<<<lutg, 256, 0, s>>>(st, 1);
  // normalize_data: calculate_stddev (mean pass, variance pass)
  k_row_partials<false, false><<<rowg, kRowT, kLutSlice, s>>>(gulp, st, 0);
  k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
  k_beam_sum<false><<<st.nbeam, kBeamT, 0, s>>>(st, 0);
  k_row_partials<true, false><<<rowg, kRowT, kLutSlice, s>>>(gulp, st, 0);
  k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
  k_beam_sum<true><<<st.nbeam, kBeamT, 0, s>>>(st, 0);
  // calc_bandpass_new of the normalised data -> spectral flag
  k_build_lut<<<lutg, 256, 0, s>>>(st, 2);
  k_lane_partials<<<laneg, 256, 0, s>>>(gulp, st.lut, st.part, st.nchan, st.gulp);
  k_lane_finish<<<fin_blocks, 256, 0, s>>>(st, 1);
  if (st.nscrunch > 0) {
    count_launches(11 + extra);
    return scrunch_planes(st, gulp, plain, R, wpos, dpos, s);
  }
  // apply_scrunch(8,8,100,flag=0,ts=1): bandpass_correct ...
  k_build_lut<<<lutg, 256, 0, s>>>(st, 3);
  k_lane_partials<<<laneg, 256, 0, s>>>(gulp, st.lut, st.part, st.nchan, st.gulp);
  extra += lane_finish(st, 2, fin_blocks, s) - 1;
  k_build_lut<<<lutg, 256, 0, s>>>(st, 4);
  // ... ts_correct ...
  k_ts<<<dim3((st.gulp + kTsT - 1) / kTsT, st.nbeam), kTsT, 0, s>>>(gulp, st);
  // ... normalize_data
  k_row_partials<false, true><<<rowg, kRowT, kLutSlice, s>>>(gulp, st, 1);
  k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
  k_beam_sum<false><<<st.nbeam, kBeamT, 0, s>>>(st, 1);
  k_row_partials<true, true><<<rowg, kRowT, kLutSlice, s>>>(gulp, st, 1);
  k_row_finish<<<fin_blocks, 256, 0, s>>>(st);
  k_beam_sum<true><<<st.nbeam, kBeamT, 0, s>>>(st, 1);
  // transpose_output into the ring
  k_flag_out<<<dim3(st.nchan / kOutC, (st.gulp + kOutT - 1) / kOutT, st.nbeam), 256, 0, s>>>(gulp, st, plain,
                                                                                         R, wpos, dpos);
  count_launches(24 + extra);
  return cudaGetLastError();
}
}  // namespace

// The ring writers store 4-byte words: the ring length and every write
// position (gulp starts) are multiples of 32 samples.
cudaError_t flag_gulp(const FlagState &st, const void *gulp, uint8_t *plain, long R, long wpos,
                      cudaStream_t s) {
  if (R % 32 != 0 || wpos % 32 != 0 || st.gulp % 32 != 0) return cudaErrorInvalidValue;
  return flag_impl(st, gulp, plain, R, wpos, nullptr, s);
}

cudaError_t flag_gulp_dev(const FlagState &st, const void *gulp, uint8_t *plain, long R,
                          const GulpPos *pos, cudaStream_t s) {
  if (R % 32 != 0 || st.gulp % 32 != 0) return cudaErrorInvalidValue;
  return flag_impl(st, gulp, plain, R, 0, pos, s);
}

// ----------------------------------------------------------- self-check
namespace {

__global__ void k_fp16_selftest(unsigned long long *bad, unsigned int *first) {
  const unsigned long long n = 31744ull * 31743ull;  // a in [0, 0x7c00), b in [1, 0x7c00)
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned short ab = (unsigned short)(i / 31743ull);
    const unsigned short bb = (unsigned short)(i % 31743ull + 1);
    const __half a = __ushort_as_half(ab), b = __ushort_as_half(bb);
    const float fa = __half2float(a), fb = __half2float(b);
    bool mismatch = __half_as_ushort(__hdiv(a, b)) != __half_as_ushort(__float2half_rn(__fdiv_rn(fa, fb)));
    if ((i & 63) == 0) {
      mismatch |= __half_as_ushort(__hadd(a, b)) != __half_as_ushort(__float2half_rn(__fadd_rn(fa, fb)));
      mismatch |= __half_as_ushort(__hmul(a, b)) != __half_as_ushort(__float2half_rn(__fmul_rn(fa, fb)));
    }
    if (mismatch) {
      atomicAdd(bad, 1ull);
      atomicCAS(first, 0xffffffffu, ((unsigned int)ab << 16) | bb);
    }
  }
}

}  // namespace
}  // namespace hg

extern "C" hella_status hella_fp16_selftest(int device, unsigned long long *mismatches,
                                            uint32_t *first_bad) {
  if (!mismatches || !first_bad) return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return HELLA_ERR_CUDA;
  unsigned long long *d_bad = nullptr;
  unsigned int *d_first = nullptr;
  hella_status st = HELLA_OK;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess || cudaMalloc(&d_first, 4) != cudaSuccess) {
    st = HELLA_ERR_ALLOC;
  } else if (cudaMemset(d_bad, 0, 8) != cudaSuccess || cudaMemset(d_first, 0xff, 4) != cudaSuccess) {
    st = HELLA_ERR_CUDA;
  } else {
    hg::k_fp16_selftest<<<152 * 8, 256>>>(d_bad, d_first);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(mismatches, d_bad, 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(first_bad, d_first, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
      st = HELLA_ERR_CUDA;
  }
  cudaFree(d_bad);
  cudaFree(d_first);
  cudaGetLastError();
  return st;
}
