// dedisp.cu -- brute-force direct dedispersion on GB300 (sm_103a).
//
// Computes out[d][t] = sum over active channels c of x[c][t + delay(c,d)]
// exactly in integers, the operation casm-hella obtains from
// dedisp_execute_adv (src/hella/src/dedisperse.cpp:17-48).
//
// Operand layout.  The input ring is kept "packed": word q of a channel row
// holds the samples q, q+S, q+2S and q+3S (S = kPackS = 256) in its four
// bytes.  Thread j of a block owns the four output samples t0+j+kS (k=0..3)
// of every DM trial in the block's tile, so for channel c and trial d it
// reads the single word at t0 + j + delay(c,d): 32 lanes read 32
// consecutive words (no bank conflicts) whatever the delay, and each 4-byte
// read feeds four sums.  The bytes are split into two SWAR registers of
// 16-bit lanes with byte_perm (samples k=0,2 and k=1,3); two channels are
// added per three-input add.  256 channels of u8 fit a 16-bit lane
// (255*256 < 2^16), after which the lanes are widened into 32-bit totals.
//
// Staging.  A block owns DPT trials x 4S samples and walks the active
// channels kStageCh at a time.  Host-built tile tables give, per (tile,
// channel), the delay of the tile's first trial, the delay spread across
// the tile and the per-trial offsets, so every stage is a set of contiguous
// 16-byte copies: the channel's packed words [t0 + delay, + S + spread) and
// its offsets.  Stages are double buffered with cp.async: stage k+1 (and the
// table entries of stage k+2) stream into shared memory while stage k is
// summed.
#include "hg_internal.h"

#include <algorithm>

namespace hg {
namespace {

constexpr int S = kPackS;
constexpr int kStageCh = 8;          // channels per pipeline stage
constexpr size_t kSmemBudget = 110 * 1024;  // two resident blocks per SM

__host__ __device__ constexpr int row_words(int max_spread) {
  // sh + S + spread words (sh < 4) rounded up to 16-byte chunks
  return ((S + max_spread + 6) + 3) / 4 * 4;
}
__host__ __device__ constexpr int off_width(int dpt) { return dpt < 4 ? 4 : dpt; }

__host__ __device__ constexpr size_t stage_words(int dpt, int rowstride) {
  return (size_t)kStageCh * 4 /*meta*/ + kStageCh /*sh*/ + (size_t)kStageCh * off_width(dpt) +
         (size_t)kStageCh * rowstride;
}
size_t smem_bytes(int dpt, int rowstride) { return 2 * stage_words(dpt, rowstride) * 4 + 64; }

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int DPT>
__global__ void __launch_bounds__(kDedispThreads, 2) k_dedisp(DedispArgs a, int rowstride) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int CC = kStageCh, OFFW = off_width(DPT);
  // per buffer b: meta [CC] int4 | sh [CC] int | off [CC][OFFW] int | rows [CC][rowstride]
  const size_t sw = stage_words(DPT, rowstride);
  auto meta_of = [&](int b) { return reinterpret_cast<int4 *>(smem + b * sw); };
  auto sh_of = [&](int b) { return reinterpret_cast<int *>(smem + b * sw + CC * 4); };
  auto off_of = [&](int b) { return reinterpret_cast<int *>(smem + b * sw + CC * 5); };
  auto rows_of = [&](int b) { return smem + b * sw + CC * 5 + CC * OFFW; };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t0 = blockIdx.x * 4 * S;
  const int tile = blockIdx.y;
  const int d0 = a.dm_first + tile * DPT, dlast = a.dm_first + a.dm_count - 1;
  const int4 *gmeta = a.tile_meta + (size_t)tile * a.nact;
  const int *goff = a.tile_off + (size_t)tile * a.nact * OFFW;
  const int nstage = (a.nact + CC - 1) / CC;
  const long w0 = (a.win0 + t0) % a.R;

  auto issue_meta = [&](int st) {
    const int k0 = st * CC, nc = min(CC, a.nact - k0);
    if (tid < nc) cp_async16(meta_of(st & 1) + tid, gmeta + k0 + tid);
  };
  auto issue_data = [&](int st) {
    const int b = st & 1, k0 = st * CC, nc = min(CC, a.nact - k0);
    const int4 *m = meta_of(b);
    int *off = off_of(b);
    for (int i = tid; i < nc * OFFW / 4; i += blockDim.x) cp_async16(off + 4 * i, goff + (size_t)k0 * OFFW + 4 * i);
    uint32_t *rows = rows_of(b);
    for (int ci = warp; ci < nc; ci += blockDim.x / 32) {
      const int4 mc = m[ci];  // {channel, base delay, spread, 0}
      long p = w0 + mc.y;
      while (p >= a.R) p -= a.R;
      const long a4 = p & ~3L;
      const int sh = (int)(p - a4);
      const int n4 = (sh + S + mc.z + 3) >> 2;
      if (lane == 0) sh_of(b)[ci] = sh;
      const uint32_t *src = a.packed + (size_t)mc.x * a.R;
      uint32_t *dst = rows + (size_t)ci * rowstride;
      for (int j = lane; j < n4; j += 32) {
        long g = a4 + 4L * j;
        while (g >= a.R) g -= a.R;  // R % 4 == 0 keeps g 16-byte aligned
        cp_async16(dst + 4 * j, src + g);
      }
    }
  };

  uint32_t acc_e[DPT], acc_o[DPT], tot[DPT][4];
#pragma unroll
  for (int m = 0; m < DPT; ++m) {
    acc_e[m] = acc_o[m] = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) tot[m][k] = 0u;
  }
  int since = 0;

  issue_meta(0);
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  issue_data(0);
  if (nstage > 1) issue_meta(1);
  cp_async_commit();

  for (int st = 0; st < nstage; ++st) {
    cp_async_wait_all();
    __syncthreads();  // stage st's rows and stage st+1's table entries have landed
    if (st + 1 < nstage) {
      issue_data(st + 1);
      if (st + 2 < nstage) issue_meta(st + 2);
    }
    cp_async_commit();
    const int b = st & 1, nc = min(CC, a.nact - st * CC);
    const char *rows = reinterpret_cast<const char *>(rows_of(b) + tid);
    const int4 *off4 = reinterpret_cast<const int4 *>(off_of(b));
    const int *shs = sh_of(b);
    // offsets are byte offsets (host-scaled), so each load address is one add
    auto add_pair = [&](int ci) {
      const char *r1 = rows + ((size_t)ci * rowstride + shs[ci]) * 4;
      const char *r2 = rows + ((size_t)(ci + 1) * rowstride + shs[ci + 1]) * 4;
#pragma unroll
      for (int q = 0; q < OFFW / 4; ++q) {
        const int4 x1 = off4[ci * (OFFW / 4) + q], x2 = off4[(ci + 1) * (OFFW / 4) + q];
        const int o1[4] = {x1.x, x1.y, x1.z, x1.w}, o2[4] = {x2.x, x2.y, x2.z, x2.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int m = 4 * q + j;
          if (m < DPT) {
            const uint32_t w1 = *reinterpret_cast<const uint32_t *>(r1 + o1[j]);
            const uint32_t w2 = *reinterpret_cast<const uint32_t *>(r2 + o2[j]);
            acc_e[m] += __byte_perm(w1, 0u, 0x4240) + __byte_perm(w2, 0u, 0x4240);
            acc_o[m] += __byte_perm(w1, 0u, 0x4341) + __byte_perm(w2, 0u, 0x4341);
          }
        }
      }
    };
    auto add_one = [&](int ci) {
      const char *r1 = rows + ((size_t)ci * rowstride + shs[ci]) * 4;
#pragma unroll
      for (int q = 0; q < OFFW / 4; ++q) {
        const int4 x1 = off4[ci * (OFFW / 4) + q];
        const int o1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int m = 4 * q + j;
          if (m < DPT) {
            const uint32_t w1 = *reinterpret_cast<const uint32_t *>(r1 + o1[j]);
            acc_e[m] += __byte_perm(w1, 0u, 0x4240);
            acc_o[m] += __byte_perm(w1, 0u, 0x4341);
          }
        }
      }
    };
    if (nc == CC) {
#pragma unroll
      for (int ci = 0; ci < CC; ci += 2) add_pair(ci);
    } else {
      int ci = 0;
      for (; ci + 1 < nc; ci += 2) add_pair(ci);
      if (ci < nc) add_one(ci);
    }
    since += nc;
    if (since > 256 - CC) {
#pragma unroll
      for (int m = 0; m < DPT; ++m) {
        tot[m][0] += acc_e[m] & 0xffffu;
        tot[m][2] += acc_e[m] >> 16;
        tot[m][1] += acc_o[m] & 0xffffu;
        tot[m][3] += acc_o[m] >> 16;
        acc_e[m] = acc_o[m] = 0u;
      }
      since = 0;
    }
  }
  cp_async_wait_all();
#pragma unroll
  for (int m = 0; m < DPT; ++m) {
    tot[m][0] += acc_e[m] & 0xffffu;
    tot[m][2] += acc_e[m] >> 16;
    tot[m][1] += acc_o[m] & 0xffffu;
    tot[m][3] += acc_o[m] >> 16;
  }
#pragma unroll
  for (int m = 0; m < DPT; ++m) {
    const int d = d0 + m;
    if (d > dlast) break;
    float *o = a.out + (size_t)(d - a.dm_first) * a.out_stride;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int t = t0 + tid + k * S;
      if (t < a.nout) o[t] = (float)tot[m][k];
    }
  }
}

__global__ void k_pack(const uint8_t *__restrict__ plain, uint32_t *__restrict__ packed,
                       int nchan, long R, long q0, long nq) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const size_t row = ((size_t)blockIdx.z * nchan + blockIdx.y) * (size_t)R;
  const long q = (q0 + i) % R;
  const uint8_t *p = plain + row;
  const uint32_t b0 = p[q], b1 = p[(q + S) % R], b2 = p[(q + 2 * S) % R],
                 b3 = p[(q + 3 * S) % R];
  packed[row + q] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
}

// [nsamps][in_stride] -> [nchan][R], 32x32 tiles through shared memory.
__global__ void k_transpose_tf(const uint8_t *__restrict__ in, size_t in_stride,
                               int nsamps, int nchan, uint8_t *__restrict__ out, long R) {
  __shared__ uint8_t tile[32][33];
  const int c0 = blockIdx.x * 32, t0 = blockIdx.y * 32, tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int t = t0 + ty + j, c = c0 + tx;
    tile[ty + j][tx] = (t < nsamps && c < nchan) ? in[(size_t)t * in_stride + c] : 0;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int c = c0 + ty + j, t = t0 + tx;
    if (c < nchan && t < R) out[(size_t)c * R + t] = tile[tx][ty + j];
  }
}

}  // namespace

DedispTables dedisp_tables(const int *delays, int nchan, const int *chans, int nact, int dm_first,
                           int dm_count) {
  DedispTables t;
  const int dlast = dm_first + dm_count - 1;
  for (int dpt : {16, 8, 4, 2, 1}) {
    int spread = 0;
    for (int d0 = dm_first; d0 <= dlast; d0 += dpt) {
      const int d1 = std::min(d0 + dpt - 1, dlast);
      for (int k = 0; k < nact; ++k) {
        const int c = chans[k];
        spread = std::max(spread, delays[(size_t)d1 * nchan + c] - delays[(size_t)d0 * nchan + c]);
      }
    }
    if (smem_bytes(dpt, row_words(spread)) <= kSmemBudget || dpt == 1) {
      t.dpt = dpt;
      t.max_spread = spread;
      break;
    }
  }
  t.offw = off_width(t.dpt);
  t.ntiles = (dm_count + t.dpt - 1) / t.dpt;
  t.meta.resize((size_t)t.ntiles * nact);
  t.off.assign((size_t)t.ntiles * nact * t.offw, 0);
  for (int i = 0; i < t.ntiles; ++i) {
    const int d0 = dm_first + i * t.dpt, d1 = std::min(d0 + t.dpt - 1, dlast);
    for (int k = 0; k < nact; ++k) {
      const int c = chans[k];
      const int base = delays[(size_t)d0 * nchan + c];
      t.meta[(size_t)i * nact + k] = make_int4(c, base, delays[(size_t)d1 * nchan + c] - base, 0);
      int *o = &t.off[((size_t)i * nact + k) * t.offw];
      for (int m = 0; m < t.dpt; ++m)  // byte offsets into the staged row
        o[m] = 4 * (delays[(size_t)std::min(d0 + m, dlast) * nchan + c] - base);
    }
  }
  return t;
}

namespace {

template <int DPT>
cudaError_t launch(const DedispArgs &a, cudaStream_t s) {
  const int rowstride = row_words(a.max_spread);
  const size_t smem = smem_bytes(DPT, rowstride);
  auto kern = k_dedisp<DPT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((a.nout + 4 * S - 1) / (4 * S), (a.dm_count + DPT - 1) / DPT);
  kern<<<grid, kDedispThreads, smem, s>>>(a, rowstride);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t dedisperse(const DedispArgs &a, cudaStream_t s) {
  if (a.dm_count <= 0 || a.nout <= 0 || a.nact <= 0) return cudaSuccess;
  switch (a.dpt) {
    case 16: return launch<16>(a, s);
    case 8: return launch<8>(a, s);
    case 4: return launch<4>(a, s);
    case 2: return launch<2>(a, s);
    case 1: return launch<1>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t pack_ring(const uint8_t *plain, uint32_t *packed, int nbeam, int nchan,
                      long R, long q0, long nq, cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  q0 = ((q0 % R) + R) % R;
  nq = std::min(nq, R);  // each ring position once
  const dim3 grid((unsigned)((nq + 255) / 256), nchan, nbeam);
  k_pack<<<grid, 256, 0, s>>>(plain, packed, nchan, R, q0, nq);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t transpose_tf(const uint8_t *in, size_t in_stride, int nsamps, int nchan,
                         uint8_t *plain, long R, cudaStream_t s) {
  const dim3 grid((nchan + 31) / 32, (unsigned)((R + 31) / 32));
  k_transpose_tf<<<grid, dim3(32, 8), 0, s>>>(in, in_stride, nsamps, nchan, plain, R);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg

// ------------------------------------------------------ measurement helpers
#include "hella_search.h"

#include <atomic>

namespace hg {
namespace {
std::atomic<unsigned long long> g_launches{0};

// Four independent coupled pairs per thread (x += y; y += x), which no
// compiler folds into fewer adds; the result is stored so the chains stay.
__global__ void k_int_add_peak(unsigned *out, int iters, unsigned seed) {
  unsigned x0 = seed ^ threadIdx.x, y0 = x0 * 3u, x1 = x0 * 5u, y1 = x0 * 7u, x2 = x0 * 11u,
           y2 = x0 * 13u, x3 = x0 * 17u, y3 = blockIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 += y0; y0 += x0; x1 += y1; y1 += x1; x2 += y2; y2 += x2; x3 += y3; y3 += x3;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 ^ y0 ^ x1 ^ y1 ^ x2 ^ y2 ^ x3 ^ y3;
}
}  // namespace

void count_launches(unsigned n) { g_launches += n; }
}  // namespace hg

extern "C" unsigned long long hella_kernel_launches(void) { return hg::g_launches.load(); }

extern "C" hella_status hella_int_add_peak(int device, double *adds_per_s) {
  if (!adds_per_s) return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return HELLA_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  unsigned *out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, (size_t)blocks * threads * 4) != cudaSuccess) return HELLA_ERR_ALLOC;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    hg::k_int_add_peak<<<blocks, threads>>>(out, iters, 12345u + rep);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  const hella_status st = cudaGetLastError() == cudaSuccess ? HELLA_OK : HELLA_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *adds_per_s = (double)blocks * threads * iters * 16 * 8 / (best * 1e-3);
  return st;
}
