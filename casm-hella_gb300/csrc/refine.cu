// refine.cu -- differentiable candidate refinement (include/hella_refine.h).
//
// One fused pass per call over the cutouts: every element's model value is
// recomputed from theta (a Gaussian at the channel's fractional delay), so
// the pass reads each cutout once and writes nothing per element; it is
// bound by HBM (4 bytes per element read).  Per channel a warp accumulates
//   S0 = sum r^2,  S1 = sum r e,  S2 = sum r e u,  S3 = sum r e u^2
// (r = d - m, e = exp(-u^2/2)), from which the adjoint of chi2 follows:
//   d chi2/d amp   = -2 sum_c s_c S1        (s_c = (f_c/f0)^index)
//   d chi2/d index = -2 sum_c amp s_c ln(f_c/f0) S1
//   d chi2/d t0    = -2 sum_c amp s_c S2 / sigma
//   d chi2/d dm    = -2 sum_c tab_c amp s_c S2 / sigma
//   d chi2/d width = -2 sum_c amp s_c S3 / sigma * dsigma/dwidth
// Blocks write per-(cutout, channel group) partials; a second kernel adds
// them in a fixed order (deterministic results) and applies the forward
// output, the adjoint scaling or an Adam step.
#include "hella_refine.h"
#include "hg_internal.h"
#include "hg_plan.h"

#include <cmath>
#include <cstdint>
#include <new>
#include <vector>

namespace {

constexpr int kWarps = 8;
constexpr int kChPerWarp = 2;
constexpr int kChPerBlock = kWarps * kChPerWarp;
constexpr int kNp = 6;  // chi2 + 5 gradient partials
constexpr int kLoads = 8;  // float4 loads per lane per round

struct RefineArgs {
  const float *cut;     // [n][nchan][nsamp]
  const float *dm_ref;  // [n]
  const float *theta;   // [n][5]
  const float *tab;     // [nchan] delay per unit DM, samples
  const float *lnf;     // [nchan] ln(f_c / f0)
  int nchan, nsamp, nblk;
  float c_w;            // sigma (samples) per ms of FWHM
  float *part;          // [n][nblk][kNp]
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <bool GRAD>
__global__ void __launch_bounds__(kWarps * 32) k_refine(RefineArgs a) {
  __shared__ float red[kWarps][kNp];
  const int i = blockIdx.y, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float *th = a.theta + (size_t)i * HELLA_REFINE_NPAR;
  const float dm = th[0], t0 = th[1], amp = th[3], idx = th[4];
  const float sigma = __fmul_rn(th[2], a.c_w);
  const float inv = __frcp_rn(sigma);
  const float dmr = a.dm_ref[i];
  float acc[kNp] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int j = 0; j < kChPerWarp; ++j) {
    const int c = blockIdx.x * kChPerBlock + warp * kChPerWarp + j;
    if (c >= a.nchan) break;
    const float tb = a.tab[c];
    const int off = (int)__fadd_rn(__fmul_rn(dmr, tb), 0.5f);  // the plan's integer delay
    // mu = t0 + dm*tab - off, formed without cancelling two large delays:
    // (dm - dm_ref)*tab is small, and dm_ref*tab - off is rounded once
    const float res = __fmaf_rn(dmr, tb, -(float)off);
    const float mu = __fadd_rn(__fmaf_rn(__fsub_rn(dm, dmr), tb, t0), res);
    const float s = expf(__fmul_rn(idx, a.lnf[c]));
    const float sc = __fmul_rn(amp, s);
    const float b = __fmul_rn(-mu, inv);
    const float4 *row = reinterpret_cast<const float4 *>(a.cut + ((size_t)i * a.nchan + c) * a.nsamp);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    const int nq = a.nsamp / 4;
    for (int q0 = lane; q0 < nq; q0 += 32 * kLoads) {
      float4 d4[kLoads];  // kLoads independent 16-byte loads in flight per lane
#pragma unroll
      for (int l = 0; l < kLoads; ++l)
        d4[l] = q0 + 32 * l < nq ? __ldcs(row + q0 + 32 * l) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int l = 0; l < kLoads; ++l) {
        const int q = q0 + 32 * l;
        if (q >= nq) break;
        const float dv[4] = {d4[l].x, d4[l].y, d4[l].z, d4[l].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float u = __fmaf_rn((float)(4 * q + k), inv, b);
          const float e = exp2f(__fmul_rn(-0.72134752f, __fmul_rn(u, u)));  // exp(-u^2/2)
          const float r = __fsub_rn(dv[k], __fmul_rn(sc, e));
          s0 = __fmaf_rn(r, r, s0);
          if (GRAD) {
            const float re = __fmul_rn(r, e);
            s1 = __fadd_rn(s1, re);
            s2 = __fmaf_rn(re, u, s2);
            s3 = __fmaf_rn(__fmul_rn(re, u), u, s3);
          }
        }
      }
    }
    s0 = warp_sum(s0);
    acc[0] = __fadd_rn(acc[0], s0);
    if (GRAD) {
      s1 = warp_sum(s1);
      s2 = warp_sum(s2);
      s3 = warp_sum(s3);
      const float gmu = __fmul_rn(__fmul_rn(-2.f, sc), __fmul_rn(inv, s2));
      acc[1] = __fmaf_rn(tb, gmu, acc[1]);                                     // dm
      acc[2] = __fadd_rn(acc[2], gmu);                                         // t0
      acc[3] = __fadd_rn(acc[3], __fmul_rn(__fmul_rn(-2.f, sc), __fmul_rn(__fmul_rn(inv, a.c_w), s3)));  // width
      acc[4] = __fadd_rn(acc[4], __fmul_rn(__fmul_rn(-2.f, s), s1));           // amp
      acc[5] = __fadd_rn(acc[5], __fmul_rn(__fmul_rn(-2.f, __fmul_rn(sc, a.lnf[c])), s1));  // index
    }
  }
  if (lane == 0)
    for (int k = 0; k < kNp; ++k) red[warp][k] = acc[k];
  __syncthreads();
  if (tid < kNp) {
    float v = 0.f;
    for (int w = 0; w < kWarps; ++w) v = __fadd_rn(v, red[w][tid]);
    a.part[((size_t)i * a.nblk + blockIdx.x) * kNp + tid] = v;
  }
}

struct Adam {
  float *m, *v;        // [n][5]
  float lr[HELLA_REFINE_NPAR];
  float bc1, bc2;      // 1 - beta^t
};

// MODE 0: chi2; 1: gtheta = gchi2 * grad; 2: chi2 and one Adam step.
template <int MODE>
__global__ void k_refine_reduce(const float *part, int n, int nblk, float *chi2, const float *gchi2,
                                float *gtheta, float *theta, Adam ad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s[kNp] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int b = 0; b < nblk; ++b)
    for (int k = 0; k < (MODE == 0 ? 1 : kNp); ++k) s[k] = __fadd_rn(s[k], part[((size_t)i * nblk + b) * kNp + k]);
  if (MODE != 1 && chi2) chi2[i] = s[0];
  // gradient order of theta: dm, t0, width, amp, index
  const float g[HELLA_REFINE_NPAR] = {s[1], s[2], s[3], s[4], s[5]};
  if (MODE == 1) {
    for (int k = 0; k < HELLA_REFINE_NPAR; ++k) gtheta[(size_t)i * HELLA_REFINE_NPAR + k] = __fmul_rn(gchi2[i], g[k]);
  } else if (MODE == 2) {
    for (int k = 0; k < HELLA_REFINE_NPAR; ++k) {
      const size_t j = (size_t)i * HELLA_REFINE_NPAR + k;
      const float m = __fmaf_rn(0.9f, ad.m[j], __fmul_rn(0.1f, g[k]));
      const float v = __fmaf_rn(0.999f, ad.v[j], __fmul_rn(0.001f, __fmul_rn(g[k], g[k])));
      ad.m[j] = m;
      ad.v[j] = v;
      const float step = __fdiv_rn(__fmul_rn(ad.lr[k], __fdiv_rn(m, ad.bc1)),
                                   __fadd_rn(__fsqrt_rn(__fdiv_rn(v, ad.bc2)), 1e-8f));
      float t = __fsub_rn(theta[j], step);
      if (k == 0) t = fmaxf(t, 0.f);     // dm
      if (k == 2) t = fmaxf(t, 0.05f);   // width, ms
      theta[j] = t;
    }
  }
}

}  // namespace

struct hella_refine {
  hella_refine_params p{};
  cudaStream_t stream = nullptr;
  int nblk = 0;
  std::vector<float> tab;
  float *d_tab = nullptr, *d_lnf = nullptr, *d_part = nullptr, *d_m = nullptr, *d_v = nullptr;
  float c_w = 0.f;
};

namespace {

hella_status check_ptrs(const hella_refine *r, int n, const float *cut, const float *dm_ref, const float *theta) {
  if (!r || !cut || !dm_ref || !theta || n < 1 || n > r->p.ncut) return HELLA_ERR_INVALID_ARG;
  if (reinterpret_cast<uintptr_t>(cut) % 16) return HELLA_ERR_INVALID_ARG;  // float4 rows
  return HELLA_OK;
}

RefineArgs args(hella_refine *r, const float *cut, const float *dm_ref, const float *theta) {
  RefineArgs a{};
  a.cut = cut;
  a.dm_ref = dm_ref;
  a.theta = theta;
  a.tab = r->d_tab;
  a.lnf = r->d_lnf;
  a.nchan = r->p.nchan;
  a.nsamp = r->p.nsamp;
  a.nblk = r->nblk;
  a.c_w = r->c_w;
  a.part = r->d_part;
  return a;
}

}  // namespace

extern "C" {

void hella_refine_destroy(hella_refine *r) {
  if (!r) return;
  cudaSetDevice(r->p.device);
  cudaStreamSynchronize(r->stream);
  cudaFree(r->d_tab);
  cudaFree(r->d_lnf);
  cudaFree(r->d_part);
  cudaFree(r->d_m);
  cudaFree(r->d_v);
  delete r;
}

hella_status hella_refine_create(hella_refine **out, const hella_refine_params *p) {
  if (!out || !p) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  if (p->ncut < 1 || p->nchan < 16 || p->nchan % kChPerBlock || p->nsamp < 128 || p->nsamp % 128 ||
      !(p->tsamp > 0) || !(p->f0_mhz > 0) || !(p->df_mhz != 0) ||
      p->f0_mhz - p->nchan * std::fabs(p->df_mhz) <= 0)
    return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(p->device) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  hella_refine *r = new (std::nothrow) hella_refine;
  if (!r) return HELLA_ERR_ALLOC;
  r->p = *p;
  r->nblk = p->nchan / kChPerBlock;
  r->c_w = (float)(1.0 / (2.0 * std::sqrt(2.0 * std::log(2.0)) * p->tsamp * 1e3));
  r->tab = hg::delay_table(p->nchan, p->tsamp, p->f0_mhz, p->df_mhz);
  std::vector<float> lnf(p->nchan);
  for (int c = 0; c < p->nchan; ++c) lnf[c] = (float)std::log((p->f0_mhz - c * std::fabs(p->df_mhz)) / p->f0_mhz);
  const size_t np = (size_t)p->ncut * HELLA_REFINE_NPAR;
  if (cudaMalloc(&r->d_tab, p->nchan * 4) != cudaSuccess || cudaMalloc(&r->d_lnf, p->nchan * 4) != cudaSuccess ||
      cudaMalloc(&r->d_part, (size_t)p->ncut * r->nblk * kNp * 4) != cudaSuccess ||
      cudaMalloc(&r->d_m, np * 4) != cudaSuccess || cudaMalloc(&r->d_v, np * 4) != cudaSuccess) {
    cudaGetLastError();
    hella_refine_destroy(r);
    return HELLA_ERR_ALLOC;
  }
  if (cudaMemcpy(r->d_tab, r->tab.data(), p->nchan * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(r->d_lnf, lnf.data(), p->nchan * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    hella_refine_destroy(r);
    return HELLA_ERR_CUDA;
  }
  *out = r;
  return HELLA_OK;
}

hella_status hella_refine_set_stream(hella_refine *r, void *stream) {
  if (!r) return HELLA_ERR_INVALID_ARG;
  r->stream = (cudaStream_t)stream;
  return HELLA_OK;
}

hella_status hella_refine_delay_table(const hella_refine *r, float *tab) {
  if (!r || !tab) return HELLA_ERR_INVALID_ARG;
  for (int c = 0; c < r->p.nchan; ++c) tab[c] = r->tab[c];
  return HELLA_OK;
}

hella_status hella_refine_forward(hella_refine *r, int n, const float *cut, const float *dm_ref,
                                  const float *theta, float *chi2) {
  hella_status s = check_ptrs(r, n, cut, dm_ref, theta);
  if (s != HELLA_OK || !chi2) return s != HELLA_OK ? s : HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(r->p.device) != cudaSuccess) return HELLA_ERR_CUDA;
  k_refine<false><<<dim3(r->nblk, n), kWarps * 32, 0, r->stream>>>(args(r, cut, dm_ref, theta));
  k_refine_reduce<0><<<(n + 255) / 256, 256, 0, r->stream>>>(r->d_part, n, r->nblk, chi2, nullptr, nullptr,
                                                              nullptr, Adam{});
  hg::count_launches(2);
  return cudaGetLastError() == cudaSuccess ? HELLA_OK : HELLA_ERR_CUDA;
}

hella_status hella_refine_adjoint(hella_refine *r, int n, const float *cut, const float *dm_ref,
                                  const float *theta, const float *gchi2, float *gtheta) {
  hella_status s = check_ptrs(r, n, cut, dm_ref, theta);
  if (s != HELLA_OK || !gchi2 || !gtheta) return s != HELLA_OK ? s : HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(r->p.device) != cudaSuccess) return HELLA_ERR_CUDA;
  k_refine<true><<<dim3(r->nblk, n), kWarps * 32, 0, r->stream>>>(args(r, cut, dm_ref, theta));
  k_refine_reduce<1><<<(n + 255) / 256, 256, 0, r->stream>>>(r->d_part, n, r->nblk, nullptr, gchi2, gtheta,
                                                              nullptr, Adam{});
  hg::count_launches(2);
  return cudaGetLastError() == cudaSuccess ? HELLA_OK : HELLA_ERR_CUDA;
}

hella_status hella_refine_fit(hella_refine *r, int n, const float *cut, const float *dm_ref, float *theta,
                              int steps, const float *lr, float *chi2) {
  hella_status s = check_ptrs(r, n, cut, dm_ref, theta);
  if (s != HELLA_OK || !lr || steps < 0) return s != HELLA_OK ? s : HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(r->p.device) != cudaSuccess) return HELLA_ERR_CUDA;
  const size_t np = (size_t)n * HELLA_REFINE_NPAR * 4;
  if (cudaMemsetAsync(r->d_m, 0, np, r->stream) != cudaSuccess ||
      cudaMemsetAsync(r->d_v, 0, np, r->stream) != cudaSuccess) {
    cudaGetLastError();
    return HELLA_ERR_CUDA;
  }
  Adam ad{r->d_m, r->d_v, {}, 0.f, 0.f};
  for (int k = 0; k < HELLA_REFINE_NPAR; ++k) ad.lr[k] = lr[k];
  double b1 = 1.0, b2 = 1.0;
  for (int t = 1; t <= steps; ++t) {
    b1 *= 0.9;
    b2 *= 0.999;
    ad.bc1 = (float)(1.0 - b1);
    ad.bc2 = (float)(1.0 - b2);
    k_refine<true><<<dim3(r->nblk, n), kWarps * 32, 0, r->stream>>>(args(r, cut, dm_ref, theta));
    k_refine_reduce<2><<<(n + 255) / 256, 256, 0, r->stream>>>(r->d_part, n, r->nblk, chi2, nullptr, nullptr,
                                                                theta, ad);
  }
  hg::count_launches(2u * steps);
  return cudaGetLastError() == cudaSuccess ? HELLA_OK : HELLA_ERR_CUDA;
}

}  // extern "C"
