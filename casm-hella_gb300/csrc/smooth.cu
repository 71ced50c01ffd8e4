// smooth.cu -- casm-hella's smoothing, per-width normalisation and peak
// finding on GB300.
//
// Reference: src/hella/src/smooth.cpp:21-127 and src/hella/src/peaks.cu:
// 31-117.  For every width sm = wmin*2^k < wmax the reference filters the
// dedispersed plane with a 3 x (2sm+1) kernel (DM weights 0.3/1/0.3 times
// time taps v(u)^2, normalised to sum 1), crops rows 1..ndms-2 and columns
// wmax/2 .. wmax/2+gulp, and standardises each width with
// calculate_stddev (normalization.cu:125-162).  find_peaks takes sigma of
// the standardised width-0 plane, gates the beam on 0.1 < sigma < 5 and
// emits every sample above snr*sigma in (width, DM row, time) order.
//
// Arithmetic (the oracle follows it operation for operation):
//   y[x]   = fmaf(0.3f, dd[r][x] + dd[r+2][x], dd[r+1][x])  (exact sum)
//   out[j] = fmaf chain over k = 0..2sm of tap[k] * y[clamp(x0 + k)]
// i.e. the DM weights factored out of the 2-D kernel, whose middle row
// supplies the time taps.  Borders replicate (NPP_BORDER_REPLICATE).
//
// Kernels.  The FIR stages a row's y values chunk by chunk in shared memory
// in a 16-phase layout, so that each thread keeps a sliding window of 16
// outputs in registers and reads one shared word per tap for all 16; every
// width is produced from the same staged chunk, and the row-mean partials
// of the reference's order (thread j sums columns j, j+256, ...) are
// accumulated as the chunk is written, so the plane is written once and
// read once more for the variance.  k_firR (spans up to 2048 samples) does
// this with constant-offset window loads and two width groups per row;
// k_fir, with runtime window addresses, takes wider spans.  Row maxima let
// the peak pass skip rows that cannot hold a candidate.
#include "hg_internal.h"

#include <algorithm>

namespace hg {
namespace {

constexpr int kR = 16;            // outputs per thread (taps padded to kR)
constexpr int kT = 256;           // threads per row block
constexpr int kCH = kR * kT;      // outputs per chunk

__device__ __forceinline__ float block256_tree(const float *p) {
  // p: 256 partials in shared memory; called by one whole warp, returns in
  // its lane 0 the total the reference's thread 0 forms (normalization.cu:
  // 41-68: each warp's shuffle tree, then the warp totals in order).
  const int lane = threadIdx.x & 31;
  float tot = 0.f;
  for (int wi = 0; wi < 8; ++wi) {
    float v = p[wi * 32 + lane];
    for (int off = 16; off > 0; off /= 2) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
    tot = wi == 0 ? v : __fadd_rn(tot, v);
  }
  return tot;
}

__device__ __forceinline__ float normv(float x, const float *st) {
  // smooth.cpp:105-123: skipped when std <= 0; else AddC(-mean), MulC(1/std)
  return st[1] > 0.f ? __fmul_rn(__fadd_rn(x, st[2]), st[3]) : x;
}

// Beam and beam-local row of global row `gr` of a launch.
__device__ __forceinline__ const SmoothBeam &row_beam(const SmoothArgs &a, int gr, int *r) {
  const SmoothBeam &B = a.beams[a.row_beam[gr]];
  *r = gr - B.row0;
  return B;
}

// One block per (beam, row): widths w0..w0+nw-1 of the row from one staged
// chunk of y values.  taps of those widths are copied to shared memory.
__global__ void __launch_bounds__(kT) k_fir(SmoothArgs a) {
  extern __shared__ __align__(16) float sm[];
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  if (!*B.active) return;
  const int w0 = a.w0, nw = a.nw, h = B.h, tid = threadIdx.x;
  const int span = 2 * (a.wmin << (w0 + nw - 1));
  const int ylen = kCH + span + 2 * kR;
  const int M = (ylen + kR - 1) / kR;
  const int tap0 = a.tap_off[w0];
  int ntaps_total = 0;
  for (int b = w0; b < w0 + nw; ++b) ntaps_total += a.tap_n[b];
  float *taps = sm;
  float *Y = taps + ((ntaps_total + 3) / 4) * 4;
  float *out_s = Y + kR * M;
  float *part_s = out_s + kCH;
  float *max_s = part_s + nw * kT;
  for (int i = tid; i < ntaps_total; i += kT) taps[i] = a.taps[tap0 + i];
  for (int j = 0; j < nw; ++j) {
    part_s[j * kT + tid] = 0.f;
    max_s[j * kT + tid] = -INFINITY;
  }
  const float *ra = B.dd + (size_t)r * B.dd_stride;
  const float *rb = ra + B.dd_stride;
  const float *rc = rb + B.dd_stride;
  const int nwcol = 256 * (a.ntime_out / 256);
  const int org = a.wmax / 2 - (a.anchor ? span : 0);

  for (int cs = 0; cs < a.ntime_out; cs += kCH) {
    __syncthreads();
    for (int x = tid; x < kR * M; x += kT) {
      int col = cs + org + x;
      col = col < 0 ? 0 : (col >= a.ntime_dd ? a.ntime_dd - 1 : col);
      Y[(x % kR) * M + x / kR] = __fmaf_rn(0.3f, __fadd_rn(ra[col], rc[col]), rb[col]);
    }
    __syncthreads();
    for (int j = 0; j < nw; ++j) {
      const int b = w0 + j;
      const int smw = a.wmin << b;
      const int off = a.anchor ? span - 2 * smw : 0;
      const float *tp = taps + a.tap_off[b] - tap0;
      const int ntap = 2 * smw + 1, nblk = ntap / kR, tail = ntap - nblk * kR;
      const int base = kR * tid + off;
      // win[] slides over y; pre[kk] is where the slot refilled at tap kk of
      // the first block of kR taps lives in Y (later blocks add one column)
      float acc[kR], win[kR];
      int pre[kR];
#pragma unroll
      for (int i = 0; i < kR; ++i) {
        acc[i] = 0.f;
        const int x = base + i, xr = base + i + kR;
        win[i] = Y[(x % kR) * M + x / kR];
        pre[i] = (xr % kR) * M + xr / kR;
      }
      int kq = 0;
      for (; kq < nblk; ++kq) {
#pragma unroll
        for (int k4 = 0; k4 < kR; k4 += 4) {
          const float4 c4 = *reinterpret_cast<const float4 *>(tp + kq * kR + k4);
          const float cfs[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int kk = k4 + jj;
#pragma unroll
            for (int i = 0; i < kR; ++i) acc[i] = __fmaf_rn(cfs[jj], win[(i + kk) % kR], acc[i]);
            win[kk] = Y[pre[kk] + kq];
          }
        }
      }
      // the last partial block: the same steps, stopping after `tail` taps
      // (no zero taps are issued; every width of 17 taps or more has a
      // 1-tap tail)
      if (tail) {
#pragma unroll
        for (int k4 = 0; k4 < kR; k4 += 4) {
          if (k4 >= tail) break;
          const float4 c4 = *reinterpret_cast<const float4 *>(tp + kq * kR + k4);
          const float cfs[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int kk = k4 + jj;
            if (kk >= tail) break;
#pragma unroll
            for (int i = 0; i < kR; ++i) acc[i] = __fmaf_rn(cfs[jj], win[(i + kk) % kR], acc[i]);
            win[kk] = Y[pre[kk] + kq];
          }
        }
      }
      float4 *o4 = reinterpret_cast<float4 *>(out_s + kR * tid);
#pragma unroll
      for (int i = 0; i < kR / 4; ++i) o4[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
      __syncthreads();
      float *dst = B.boxes + ((size_t)j * h + r) * a.ntime_out;
      float ps = part_s[j * kT + tid], mx = max_s[j * kT + tid];
#pragma unroll
      for (int m = 0; m < kR; ++m) {
        const int jc = tid + kT * m, col = cs + jc;
        if (col < a.ntime_out) {
          const float v = out_s[jc];
          dst[col] = v;
          mx = fmaxf(mx, v);
          if (col < nwcol) ps = __fadd_rn(ps, v);
        }
      }
      part_s[j * kT + tid] = ps;
      max_s[j * kT + tid] = mx;
      __syncthreads();
    }
  }
  __syncthreads();
  for (int j = tid >> 5; j < nw; j += kT / 32) {
    const float tot = block256_tree(part_s + j * kT);
    float mx = -INFINITY;
    for (int i = threadIdx.x & 31; i < kT; i += 32) mx = fmaxf(mx, max_s[j * kT + i]);
    for (int off = 16; off > 0; off /= 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((tid & 31) == 0) {
      B.rowmean[(size_t)(w0 + j) * h + r] = __fdiv_rn(tot, (float)nwcol);
      B.rowmax[(size_t)(w0 + j) * h + r] = mx;
    }
  }
}

// k_firR: the arithmetic of k_fir with R outputs per thread (R = 16 or
// 32) and 128 threads per (row, width group); widths [w0, split) form
// group 0 and [split, w0 + nw) group 1 (blockIdx.y), so that a short list
// of long rows still fills the GPU.  The chunk's y values are staged in an
// R-phase layout with a compile-time phase stride M and 2R phase rows,
//   Y[p * M + c] = y(R c + p)   (p < 2R, c < M),
// so that for every width (off = R O + o) window element n of thread t is
// Y[(o + n % R) * M + t + O + n / R]: one base address per width, and
// every load of the tap loop sits at a constant offset from it.  Outputs
// go to global memory straight from registers; the row-mean partials of
// the reference's order (owner j sums columns j, j + 256, ...) read them
// back through a swizzled shared transpose (conflict-free both ways).
constexpr int kTF = 128;  // threads per block

// float4 slot q of thread t's R outputs sits at slot q ^ fir_swz_key(t).
template <int R>
__device__ __forceinline__ int fir_swz_key(int t) {
  return R == 32 ? (t & 7) : ((t >> 1) & 3);
}
// Transposed position of chunk column c.
template <int R>
__device__ __forceinline__ int fir_swz(int c) {
  const int t = c / R, q = (c % R) >> 2;
  return R * t + 4 * (q ^ fir_swz_key<R>(t)) + (c & 3);
}

template <int R, int M>
__global__ void __launch_bounds__(kTF, R == 32 ? 3 : 5) k_firR(SmoothArgs a) {
  constexpr int kC = R * kTF;  // outputs per chunk
  extern __shared__ __align__(16) float sm[];
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  if (!*B.active) return;
  const int wb = blockIdx.y == 0 ? a.w0 : a.split, we = blockIdx.y == 0 ? a.split : a.w0 + a.nw;
  const int nw = we - wb;
  if (nw <= 0) return;
  const int h = B.h, tid = threadIdx.x;
  const int span = 2 * (a.wmin << (a.w0 + a.nw - 1));
  const int tap0 = a.tap_off[wb];
  int ntaps_total = 0;
  for (int b = wb; b < we; ++b) ntaps_total += a.tap_n[b];
  float *taps = sm;
  float *Y = taps + ((ntaps_total + 3) / 4) * 4;
  float *out_s = Y + 2 * R * M;
  float *part_s = out_s + kC;        // [nw][256] row-mean partials
  float *max_s = part_s + nw * 256;  // [nw][kTF] row maxima
  for (int i = tid; i < ntaps_total; i += kTF) taps[i] = a.taps[tap0 + i];
  for (int j = 0; j < nw; ++j) {
    part_s[j * 256 + tid] = 0.f;
    part_s[j * 256 + kTF + tid] = 0.f;
    max_s[j * kTF + tid] = -INFINITY;
  }
  const float *ra = B.dd + (size_t)r * B.dd_stride;
  const float *rb = ra + B.dd_stride;
  const float *rc = rb + B.dd_stride;
  const int nwcol = 256 * (a.ntime_out / 256);
  const int org = a.wmax / 2 - (a.anchor ? span : 0);

  constexpr int NY = R * (M + 1);                // staged y values
  constexpr int NX = (NY + kTF - 1) / kTF;       // per thread
  constexpr int XB = 6;                          // loads in flight per thread
  for (int cs = 0; cs < a.ntime_out; cs += kC) {
    __syncthreads();
    for (int i0 = 0; i0 < NX; i0 += XB) {
      float va[XB], vb[XB], vc[XB];
#pragma unroll
      for (int u = 0; u < XB; ++u) {
        int col = cs + org + tid + (i0 + u) * kTF;
        col = col < 0 ? 0 : (col >= a.ntime_dd ? a.ntime_dd - 1 : col);
        va[u] = ra[col];
        vb[u] = rb[col];
        vc[u] = rc[col];
      }
#pragma unroll
      for (int u = 0; u < XB; ++u) {
        const int x = tid + (i0 + u) * kTF;
        const int c = x / R, p = x % R;
        if (x < NY) {
          const float y = __fmaf_rn(0.3f, __fadd_rn(va[u], vc[u]), vb[u]);
          if (c < M) Y[p * M + c] = y;
          if (c >= 1) Y[(p + R) * M + c - 1] = y;
        }
      }
    }
    __syncthreads();
    const bool valid = cs + R * tid < a.ntime_out;  // ntime_out % R == 0
    for (int j = 0; j < nw; ++j) {
      const int b = wb + j;
      const int smw = a.wmin << b;
      const int off = a.anchor ? span - 2 * smw : 0;
      const float *tp = taps + a.tap_off[b] - tap0;
      const int ntap = 2 * smw + 1, nblk = ntap / R, tail = ntap % R;
      const float *Yp = Y + (off % R) * M + tid + off / R;
      // win[(i + kk) % R] holds y at window element R kq + kk + i of output
      // i; slot kk is refilled after step kk of block kq
      float acc[R], win[R];
#pragma unroll
      for (int i = 0; i < R; ++i) {
        acc[i] = 0.f;
        win[i] = Yp[i * M];
      }
      // taps are read one group of four ahead (cn); ntap is odd, so the
      // group after the last full block is the tail's first
      float4 cn = *reinterpret_cast<const float4 *>(tp);
      int kq = 0;
      for (; kq < nblk; ++kq) {
        const float *Yq = Yp + kq + 1;
        const float *tq = tp + kq * R;
#pragma unroll
        for (int k4 = 0; k4 < R; k4 += 4) {
          const float4 c4 = cn;
          cn = *reinterpret_cast<const float4 *>(tq + k4 + 4);
          const float cfs[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int kk = k4 + jj;
#pragma unroll
            for (int i = 0; i < R; ++i) acc[i] = __fmaf_rn(cfs[jj], win[(i + kk) % R], acc[i]);
            win[kk] = Yq[kk * M];
          }
        }
      }
      if (tail) {  // the last `tail` taps (no zero taps are issued)
        const float *Yq = Yp + kq + 1;
        const float *tq = tp + kq * R;
#pragma unroll
        for (int k4 = 0; k4 < R; k4 += 4) {
          if (k4 >= tail) break;
          const float4 c4 = cn;
          if (k4 + 4 < tail) cn = *reinterpret_cast<const float4 *>(tq + k4 + 4);
          const float cfs[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int kk = k4 + jj;
            if (kk >= tail) break;
#pragma unroll
            for (int i = 0; i < R; ++i) acc[i] = __fmaf_rn(cfs[jj], win[(i + kk) % R], acc[i]);
            win[kk] = Yq[kk * M];
          }
        }
      }
      if (valid) {
        float4 *dst = reinterpret_cast<float4 *>(B.boxes + ((size_t)(b - a.w0) * h + r) * a.ntime_out + cs +
                                                 R * tid);
        float mx = max_s[j * kTF + tid];
#pragma unroll
        for (int q = 0; q < R / 4; ++q) {
          dst[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
          mx = fmaxf(fmaxf(fmaxf(mx, acc[4 * q]), fmaxf(acc[4 * q + 1], acc[4 * q + 2])), acc[4 * q + 3]);
        }
        max_s[j * kTF + tid] = mx;
      }
      const int key = fir_swz_key<R>(tid);
#pragma unroll
      for (int q = 0; q < R / 4; ++q)
        *reinterpret_cast<float4 *>(out_s + R * tid + 4 * (q ^ key)) =
            make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
      __syncthreads();
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int jo = tid + kTF * hh, c0 = cs + jo;
        const int nm = c0 < nwcol ? min(kC / 256, (nwcol - c0 + 255) >> 8) : 0;
        const float *src = out_s + fir_swz<R>(jo);  // column jo + 256 m at src[256 m]
        float ps = part_s[j * 256 + jo];
#pragma unroll
        for (int m = 0; m < kC / 256; ++m)
          if (m < nm) ps = __fadd_rn(ps, src[256 * m]);
        part_s[j * 256 + jo] = ps;
      }
      __syncthreads();
    }
  }
  for (int j = tid >> 5; j < nw; j += kTF / 32) {
    const float tot = block256_tree(part_s + j * 256);
    float mx = -INFINITY;
    for (int i = threadIdx.x & 31; i < kTF; i += 32) mx = fmaxf(mx, max_s[j * kTF + i]);
    for (int o = 16; o > 0; o /= 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) {
      B.rowmean[(size_t)(wb + j) * h + r] = __fdiv_rn(tot, (float)nwcol);
      B.rowmax[(size_t)(wb + j) * h + r] = mx;
    }
  }
}

// k_firS: the arithmetic of k_firR for launches whose widths are all at
// most 32 (wmin 1, wmax <= 64: spans of at most 64 samples), the widths of
// the plain, batched and streaming configurations, whose few taps per width
// left k_firR's per-width window set-up, stores, transposes and barriers as
// large as the multiply-adds.  256 threads, 8 outputs each (the same
// 2048-output chunks); thread t keeps the 72 y values its outputs read in
// registers, so every tap is eight multiply-adds on registers; each width's
// outputs get their own slot of a shared buffer, so one barrier pair per
// chunk serves the row-mean partials of every width.  Per output: the same
// multiply-add chain over the taps in order from zero, the same y values
// and the same partial order as k_firR.
constexpr int kSO = 8;                  // outputs per thread
constexpr int kST = 256;                // threads per block
constexpr int kSC = kSO * kST;          // outputs per chunk (k_firR's)
constexpr int kSSpan = 64;              // largest span served
constexpr int kSW = 6;                  // widths 1, 2, 4, 8, 16, 32
constexpr int kSWin = kSO + kSSpan;     // y values a thread reads (72)
constexpr int kSY = kSC + kSSpan + kSO; // y values staged per chunk (2120)
constexpr int kSTap = 68;               // taps kept per width (65 used at most, float4 loads)
static_assert(kSWin % 4 == 0 && kSY % 4 == 0 && kSTap % 4 == 0, "float4 staging");

// One width (2 SM + 1 taps) of a thread's 8 outputs from its register window.
template <int SM, int ANCHOR>
__device__ __forceinline__ void firS_width(const float (&win)[kSWin], const float *tp, float (&acc)[kSO]) {
  constexpr int NT = 2 * SM + 1, OFF = ANCHOR ? kSSpan - 2 * SM : 0;
#pragma unroll
  for (int i = 0; i < kSO; ++i) acc[i] = 0.f;
#pragma unroll
  for (int n4 = 0; n4 < NT; n4 += 4) {
    const float4 c4 = *reinterpret_cast<const float4 *>(tp + n4);
    const float cf[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int n = n4 + jj;
      if (n < NT) {
#pragma unroll
        for (int i = 0; i < kSO; ++i) acc[i] = __fmaf_rn(cf[jj], win[OFF + i + n], acc[i]);
      }
    }
  }
}

template <int ANCHOR>
__global__ void __launch_bounds__(kST, 2) k_firS(SmoothArgs a) {
  extern __shared__ __align__(16) float sm[];
  float *Ys = sm;                     // [kSY]
  float *out_s = Ys + kSY;            // [kSW][kSC]
  float *part_s = out_s + kSW * kSC;  // [kSW][256]
  float *taps = part_s + kSW * 256;   // [kSW][kSTap]
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  if (!*B.active) return;
  const int h = B.h, tid = threadIdx.x, bw0 = a.w0, bw1 = a.w0 + a.nw;
  for (int i = tid; i < kSW * kSTap; i += kST) {
    const int b = i / kSTap, n = i - b * kSTap;
    taps[i] = b < a.nbox && n < a.tap_n[b] ? a.taps[a.tap_off[b] + n] : 0.f;
  }
  for (int i = tid; i < kSW * 256; i += kST) part_s[i] = 0.f;
  float mx[kSW];
#pragma unroll
  for (int b = 0; b < kSW; ++b) mx[b] = -INFINITY;
  const float *ra = B.dd + (size_t)r * B.dd_stride;
  const float *rb = ra + B.dd_stride;
  const float *rc = rb + B.dd_stride;
  const int nwcol = 256 * (a.ntime_out / 256);
  const int org = a.wmax / 2 - (ANCHOR ? kSSpan : 0);
  constexpr int NL = (kSY + kST - 1) / kST;  // staged values per thread
  for (int cs = 0; cs < a.ntime_out; cs += kSC) {
    __syncthreads();  // the previous chunk's shared reads are done
    {
      float va[NL], vb[NL], vc[NL];
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int sx = tid + u * kST;
        int col = cs + org + sx;
        col = col < 0 ? 0 : (col >= a.ntime_dd ? a.ntime_dd - 1 : col);
        if (sx < kSY) {
          va[u] = ra[col];
          vb[u] = rb[col];
          vc[u] = rc[col];
        }
      }
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int sx = tid + u * kST;
        if (sx < kSY) Ys[sx] = __fmaf_rn(0.3f, __fadd_rn(va[u], vc[u]), vb[u]);
      }
    }
    __syncthreads();
    float win[kSWin];
#pragma unroll
    for (int q = 0; q < kSWin / 4; ++q) {
      const float4 v = *reinterpret_cast<const float4 *>(Ys + kSO * tid + 4 * q);
      win[4 * q] = v.x;
      win[4 * q + 1] = v.y;
      win[4 * q + 2] = v.z;
      win[4 * q + 3] = v.w;
    }
    const bool valid = cs + kSO * tid < a.ntime_out;  // ntime_out % kSO == 0
    float acc[kSO];
    auto emit = [&](int b) {
      if (valid) {
        float4 *dst = reinterpret_cast<float4 *>(B.boxes + ((size_t)(b - a.w0) * h + r) * a.ntime_out + cs +
                                                 kSO * tid);
        dst[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        dst[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
#pragma unroll
        for (int i = 0; i < kSO; ++i) mx[b] = fmaxf(mx[b], acc[i]);
      }
      float4 *o = reinterpret_cast<float4 *>(out_s + b * kSC + kSO * tid);
      o[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
      o[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    };
    if (bw0 <= 0 && 0 < bw1) { firS_width<1, ANCHOR>(win, taps + 0 * kSTap, acc); emit(0); }
    if (bw0 <= 1 && 1 < bw1) { firS_width<2, ANCHOR>(win, taps + 1 * kSTap, acc); emit(1); }
    if (bw0 <= 2 && 2 < bw1) { firS_width<4, ANCHOR>(win, taps + 2 * kSTap, acc); emit(2); }
    if (bw0 <= 3 && 3 < bw1) { firS_width<8, ANCHOR>(win, taps + 3 * kSTap, acc); emit(3); }
    if (bw0 <= 4 && 4 < bw1) { firS_width<16, ANCHOR>(win, taps + 4 * kSTap, acc); emit(4); }
    if (bw0 <= 5 && 5 < bw1) { firS_width<32, ANCHOR>(win, taps + 5 * kSTap, acc); emit(5); }
    __syncthreads();
    // row-mean partials in the reference's order: owner jo adds columns jo, jo + 256, ...
    const int c0 = cs + tid;
    const int nm = c0 < nwcol ? min(kSC / 256, (nwcol - c0 + 255) >> 8) : 0;
    for (int b = bw0; b < bw1; ++b) {
      float ps = part_s[b * 256 + tid];
#pragma unroll
      for (int m = 0; m < kSC / 256; ++m)
        if (m < nm) ps = __fadd_rn(ps, out_s[b * kSC + tid + 256 * m]);
      part_s[b * 256 + tid] = ps;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < kSW; ++b)
    if (b >= bw0 && b < bw1) out_s[b * 256 + tid] = mx[b];
  __syncthreads();
  for (int b = bw0 + (tid >> 5); b < bw1; b += kST / 32) {
    const float tot = block256_tree(part_s + b * 256);
    float m = -INFINITY;
    for (int i = threadIdx.x & 31; i < kST; i += 32) m = fmaxf(m, out_s[b * 256 + i]);
    for (int o = 16; o > 0; o /= 2) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((tid & 31) == 0) {
      B.rowmean[(size_t)b * h + r] = __fdiv_rn(tot, (float)nwcol);
      B.rowmax[(size_t)b * h + r] = m;
    }
  }
}

// Sequential sum of v[0..n) in index order (the reference's host loop),
// in thread 0 of a kFin-thread block: the block stages kFinChunk values at
// a time in shared memory with coalesced loads, thread 0 adds them.
constexpr int kFin = 256, kFinChunk = 4096;
__device__ float block_seq_sum(const float *v, int n, float *chunk_s) {
  float s = 0.f;
  for (int c0 = 0; c0 < n; c0 += kFinChunk) {
    const int m = min(kFinChunk, n - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += kFin) chunk_s[i] = v[c0 + i];
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < m; ++i) s = __fadd_rn(s, chunk_s[i]);
  }
  return s;
}

// Host loop of calculate_stddev (normalization.cu:138-142): sequential over
// rows, / height.  Block = (beam, width of the launch).
__global__ void __launch_bounds__(kFin) k_mean_finish(SmoothArgs a) {
  __shared__ float chunk_s[kFinChunk];
  const SmoothBeam &B = a.beams[blockIdx.x];
  const int j = blockIdx.y;
  if (!*B.active) return;
  const int b = a.w0 + j, h = B.h;
  const float s = block_seq_sum(B.rowmean + (size_t)b * h, h, chunk_s);
  if (threadIdx.x == 0) B.stats[b * 4 + 0] = __fdiv_rn(s, (float)h);
}

// computeRowVariances over one row of one width plane.  NORM0: the
// normalised width-0 plane (find_peaks' sigma, peaks.cu:171-178), which
// needs width 0 in the launch (w0 == 0).
template <bool NORM0, bool VAR>
__global__ void __launch_bounds__(kT) k_row_stat(SmoothArgs a) {
  __shared__ float p_s[kT];
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  if (!*B.active) return;
  const int j = NORM0 ? 0 : blockIdx.y, b = a.w0 + j, h = B.h, tid = threadIdx.x;
  const float *x = B.boxes + ((size_t)j * h + r) * a.ntime_out;
  const int nwcol = 256 * (a.ntime_out / 256);
  const float *st = B.stats + b * 4;
  const float mean = NORM0 ? B.gate[0] : st[0];
  float s = 0.f;
  auto add = [&](float v) {
    if (NORM0) v = normv(v, st);
    if (VAR) {
      const float d = __fsub_rn(v, mean);
      s = __fmaf_rn(d, d, s);
    } else {
      s = __fadd_rn(s, v);
    }
  };
  // sixteen loads in flight per thread, then the sums in column order
  constexpr int kB = 16;
  int col = tid;
  for (; col + (kB - 1) * kT < nwcol; col += kB * kT) {
    float v[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) v[u] = x[col + u * kT];
#pragma unroll
    for (int u = 0; u < kB; ++u) add(v[u]);
  }
  for (; col < nwcol; col += kT) add(x[col]);
  p_s[tid] = s;
  __syncthreads();
  if (tid < 32) {
    const float tot = block256_tree(p_s);
    if (tid == 0) B.rowvar[(size_t)b * h + r] = __fdiv_rn(tot, (float)nwcol);
  }
}

// Per (beam, width): variance -> std and the normalisation constants.
// NORM0: the gate statistics of the normalised width-0 plane.
template <bool NORM0, bool VAR>
__global__ void __launch_bounds__(kFin) k_stat_finish(SmoothArgs a) {
  __shared__ float chunk_s[kFinChunk];
  const SmoothBeam &B = a.beams[blockIdx.x];
  const int j = NORM0 ? 0 : blockIdx.y;
  if (!*B.active) return;
  const int b = NORM0 ? 0 : a.w0 + j, h = B.h;
  float s = block_seq_sum(B.rowvar + (size_t)b * h, h, chunk_s);
  if (threadIdx.x != 0) return;
  s = __fdiv_rn(s, (float)h);
  if (NORM0) {
    if (!VAR) {
      B.gate[0] = s;
    } else {
      const float sig = __fsqrt_rn(s);
      B.gate[1] = sig;
      B.gate[2] = __fmul_rn(a.snr, sig);
      B.gate[3] = (a.nogate || (sig < 5 && (double)sig > 0.1)) ? 1.f : 0.f;  // definitions.h:66,71-72
    }
  } else {
    const float sd = __fsqrt_rn(s), mean = B.stats[b * 4 + 0];
    B.stats[b * 4 + 1] = sd;
    B.stats[b * 4 + 2] = -1.0f * mean;
    B.stats[b * 4 + 3] = __fdiv_rn(1.0f, sd);
  }
}

// Unnormalised planes (hella_smooth(ctx, 0)): stats zero for the widths.
__global__ void k_stat_zero(SmoothArgs a) {
  const SmoothBeam &B = a.beams[blockIdx.x];
  const int j = threadIdx.x;
  if (j >= a.nw || !*B.active) return;
  for (int q = 0; q < 4; ++q) B.stats[(a.w0 + j) * 4 + q] = 0.f;
}

__global__ void __launch_bounds__(kT) k_count(SmoothArgs a) {
  __shared__ int c_s[kT / 32];
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  const int j = blockIdx.y, b = a.w0 + j, h = B.h, tid = threadIdx.x;
  const size_t row = (size_t)b * h + r;
  const float *st = B.stats + b * 4;
  const float thr = B.gate[2];
  // normalisation is monotonic, so the row maximum decides the whole row
  if (!*B.active || B.gate[3] == 0.f || !(normv(B.rowmax[row], st) > thr)) {
    if (tid == 0) B.counts[row] = 0;
    return;
  }
  const float *x = B.boxes + ((size_t)j * h + r) * a.ntime_out;
  int n = 0;
  constexpr int kB = 16;  // loads in flight per thread
  int col = tid;
  for (; col + (kB - 1) * kT < a.ntime_out; col += kB * kT) {
    float v[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) v[u] = x[col + u * kT];
#pragma unroll
    for (int u = 0; u < kB; ++u) n += normv(v[u], st) > thr;
  }
  for (; col < a.ntime_out; col += kT) n += normv(x[col], st) > thr;
  for (int off = 16; off > 0; off /= 2) n += __shfl_xor_sync(0xffffffffu, n, off);
  if ((tid & 31) == 0) c_s[tid >> 5] = n;
  __syncthreads();
  if (tid == 0) {
    int t = 0;
    for (int i = 0; i < kT / 32; ++i) t += c_s[i];
    B.counts[row] = t;
  }
}

// Per beam: exclusive scan of the row counts of the launch's widths in
// (width, row) order, after the candidates of earlier widths; the beam's
// total is capped at its cap.
__global__ void __launch_bounds__(1024) k_scan(SmoothArgs a) {
  __shared__ int s_s[1024];
  const SmoothBeam &B = a.beams[blockIdx.x];
  if (!*B.active) return;
  const int tid = threadIdx.x;
  const int nrows = a.nw * B.h;
  int *counts = B.counts + (size_t)a.w0 * B.h, *offsets = B.offsets + (size_t)a.w0 * B.h;
  const int base = B.total[0];
  const int per = (nrows + 1023) / 1024;
  const int lo = min(nrows, tid * per), hi = min(nrows, lo + per);
  int sum = 0;
  for (int i = lo; i < hi; ++i) sum += counts[i];
  s_s[tid] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off *= 2) {
    int v = tid >= off ? s_s[tid - off] : 0;
    __syncthreads();
    s_s[tid] += v;
    __syncthreads();
  }
  int run = base + s_s[tid] - sum;
  for (int i = lo; i < hi; ++i) {
    offsets[i] = run;
    run += counts[i];
  }
  __syncthreads();
  if (tid == 1023) B.total[0] = min(base + s_s[1023], B.cap);
}

// Ordered compaction of one row's candidates, kWR chunks of 256 columns a
// round: every thread reads one column of each chunk, the warps' hit
// counts of the round are published once, and each hit is written at the
// row's offset + the hits of earlier chunks + earlier warps of its chunk +
// earlier lanes (column order).
constexpr int kWR = 4;
__global__ void __launch_bounds__(kT) k_write(SmoothArgs a) {
  __shared__ int w_s[kWR][kT / 32];
  int r;
  const SmoothBeam &B = row_beam(a, blockIdx.x, &r);
  const int j = blockIdx.y, b = a.w0 + j, h = B.h, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const size_t row = (size_t)b * h + r;
  if (!*B.active || B.counts[row] == 0 || B.offsets[row] >= B.cap) return;
  const float *st = B.stats + b * 4;
  const float thr = B.gate[2];
  const float *x = B.boxes + ((size_t)j * h + r) * a.ntime_out;
  int base = B.offsets[row];  // the same in every thread
  for (int cs = 0; cs < a.ntime_out && base < B.cap; cs += kWR * kT) {
    float v[kWR];
    unsigned bal[kWR];
#pragma unroll
    for (int m = 0; m < kWR; ++m) {
      const int col = cs + m * kT + tid;
      v[m] = col < a.ntime_out ? normv(x[col], st) : 0.f;
    }
#pragma unroll
    for (int m = 0; m < kWR; ++m) {
      const int col = cs + m * kT + tid;
      bal[m] = __ballot_sync(0xffffffffu, col < a.ntime_out && v[m] > thr);
      if (lane == 0) w_s[m][warp] = __popc(bal[m]);
    }
    __syncthreads();
    int before = base, round = 0;
#pragma unroll
    for (int m = 0; m < kWR; ++m) {
      int pos = before;
      for (int i = 0; i < kT / 32; ++i) {
        if (i == warp) pos += __popc(bal[m] & ((1u << lane) - 1u));
        const int c = w_s[m][i];
        if (i < warp) pos += c;
        round += c;
      }
      const int col = cs + m * kT + tid;
      if (((bal[m] >> lane) & 1u) && pos < B.cap) {
        B.cand_i[pos] = make_int4(B.beam_id, r + 1, b, col);
        B.cand_v[pos] = v[m];
      }
      before = base + round;
    }
    base += round;
    __syncthreads();
  }
}

// Normalised copy of beam 0's planes of the launch's widths (inspection).
__global__ void k_normalise_copy(SmoothArgs a, float *dst) {
  const SmoothBeam &B = a.beams[0];
  const size_t plane = (size_t)B.h * a.ntime_out;
  const size_t n = plane * a.nw;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = normv(B.boxes[i], B.stats + (a.w0 + i / plane) * 4);
}

}  // namespace

size_t fir_smem_bytes(const SmoothArgs &a) {
  int ntot = 0;
  for (int b = a.w0; b < a.w0 + a.nw; ++b) ntot += ((2 * (a.wmin << b) + 1 + kR - 1) / kR) * kR;
  const int span = 2 * (a.wmin << (a.w0 + a.nw - 1));
  const int ylen = kCH + span + 2 * kR;
  const int M = (ylen + kR - 1) / kR;
  return sizeof(float) * ((size_t)(ntot + 3) / 4 * 4 + (size_t)kR * M + kCH + (size_t)2 * a.nw * kT);
}

namespace {

// Outputs per thread of k_firR.
constexpr int kFirR = 16;

// Instantiated phase strides of k_firR (odd, so that staging stores of a
// warp spread over the banks): spans up to 64, 512 and 2048.
template <int R>
struct FirStrides {
  static constexpr int m0 = (129 + 65 / R) | 1, m1 = (129 + 513 / R) | 1, m2 = (129 + 2049 / R) | 1;
};
// Phase stride for the launch's span: the smallest instantiated M >= 129 +
// (span + 1) / R (the last column the tap loop reads), or 0.
template <int R>
int fir_stride(int span) {
  const int need = 129 + (span + 1) / R;
  for (int m : {FirStrides<R>::m0, FirStrides<R>::m1, FirStrides<R>::m2})
    if (need <= m) return m;
  return 0;
}

template <int R>
size_t firR_smem(const SmoothArgs &a, int M) {
  size_t best = 0;
  for (int g = 0; g < 2; ++g) {
    const int wb = g == 0 ? a.w0 : a.split, we = g == 0 ? a.split : a.w0 + a.nw;
    if (we <= wb) continue;
    int ntot = 0;
    for (int b = wb; b < we; ++b) ntot += ((2 * (a.wmin << b) + 1 + 15) / 16) * 16;
    const size_t f =
        (size_t)(ntot + 3) / 4 * 4 + (size_t)2 * R * M + (size_t)R * kTF + (size_t)(we - wb) * (256 + kTF);
    best = std::max(best, f * sizeof(float));
  }
  return best;
}

template <int R, int M>
cudaError_t launch_firR(const SmoothArgs &a, cudaStream_t s) {
  const size_t smem = firR_smem<R>(a, M);
  cudaError_t e = cudaFuncSetAttribute(k_firR<R, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_firR<R, M><<<dim3(a.nrows, a.split < a.w0 + a.nw ? 2 : 1), kTF, smem, s>>>(a);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t smooth_planes(const SmoothArgs &a0, cudaStream_t s) {
  if (a0.nrows <= 0 || a0.nw <= 0) return cudaSuccess;
  if (a0.wmin == 1 && a0.wmax <= kSSpan && a0.nbox <= kSW && a0.w0 + a0.nw <= kSW && a0.ntime_out % kSO == 0) {
    const size_t smem = sizeof(float) * ((size_t)kSY + kSW * kSC + kSW * 256 + kSW * kSTap);
    auto kern = a0.anchor ? k_firS<1> : k_firS<0>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<a0.nrows, kST, smem, s>>>(a0);
    count_launches(1);
    return cudaGetLastError();
  }
  SmoothArgs a = a0;
  a.split = a.w0 + a.nw;
  const int M = a.ntime_out % kFirR == 0 ? fir_stride<kFirR>(2 * (a.wmin << (a.w0 + a.nw - 1))) : 0;
  if (M) {
    // two width groups of about equal taps when the rows alone would leave
    // the GPU in few waves (fewer than 16 of three blocks per SM)
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return cudaErrorInvalidDevice;
    if (a.nw > 1 && a.nrows < 16 * 3 * nsm) {
      long tot = 0, run = 0, best = -1;
      for (int b = a.w0; b < a.w0 + a.nw; ++b) tot += 2 * (a.wmin << b) + 1;
      for (int b = a.w0; b < a.w0 + a.nw - 1; ++b) {
        run += 2 * (a.wmin << b) + 1;
        const long worst = std::max(run, tot - run);
        if (best < 0 || worst < best) {
          best = worst;
          a.split = b + 1;
        }
      }
    }
    using F = FirStrides<kFirR>;
    if (M == F::m0) return launch_firR<kFirR, F::m0>(a, s);
    if (M == F::m1) return launch_firR<kFirR, F::m1>(a, s);
    return launch_firR<kFirR, F::m2>(a, s);
  }
  const size_t smem = fir_smem_bytes(a);
  cudaError_t e = cudaFuncSetAttribute(k_fir, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_fir<<<a.nrows, kT, smem, s>>>(a);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t smooth_stats(const SmoothArgs &a, cudaStream_t s, int scale) {
  if (a.nrows <= 0 || a.nw <= 0) return cudaSuccess;
  unsigned n = 0;
  if (scale) {
    k_mean_finish<<<dim3(a.nbeam, a.nw), kFin, 0, s>>>(a);
    k_row_stat<false, true><<<dim3(a.nrows, a.nw), kT, 0, s>>>(a);
    k_stat_finish<false, true><<<dim3(a.nbeam, a.nw), kFin, 0, s>>>(a);
    n += 3;
  } else {
    k_stat_zero<<<a.nbeam, 32, 0, s>>>(a);
    n += 1;
  }
  if (a.w0 == 0) {  // the gate statistics of the normalised width-0 plane
    k_row_stat<true, false><<<dim3(a.nrows, 1), kT, 0, s>>>(a);
    k_stat_finish<true, false><<<a.nbeam, kFin, 0, s>>>(a);
    k_row_stat<true, true><<<dim3(a.nrows, 1), kT, 0, s>>>(a);
    k_stat_finish<true, true><<<a.nbeam, kFin, 0, s>>>(a);
    n += 4;
  }
  count_launches(n);
  return cudaGetLastError();
}

cudaError_t find_peaks(const SmoothArgs &a, cudaStream_t s) {
  if (a.nrows <= 0 || a.nw <= 0) return cudaSuccess;
  k_count<<<dim3(a.nrows, a.nw), kT, 0, s>>>(a);
  k_scan<<<a.nbeam, 1024, 0, s>>>(a);
  k_write<<<dim3(a.nrows, a.nw), kT, 0, s>>>(a);
  count_launches(3);
  return cudaGetLastError();
}

cudaError_t normalise_copy(const SmoothArgs &a, float *dst, cudaStream_t s) {
  k_normalise_copy<<<1024, 256, 0, s>>>(a, dst);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg
