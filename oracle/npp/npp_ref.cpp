// npp_ref.cpp -- TEST INFRASTRUCTURE ONLY: the two NPP filters casm-hella's
// stages call, run on the GPU as the reference runs them, so the GPU tests
// can hold this library's own filter arithmetic against the reference's.
//
//   nr_filter_f32: nppiFilterBorder_32f_C1R, the smoothing FIR
//                  (src/hella/src/smooth.cpp:61-73: a 3 x (2sm+1) kernel,
//                  anchor {0,1}, replicate border, over [ndms][ntime_dd]);
//   nr_filter_f16: nppiFilterBorder32f_16f_C1R, the SCRUNCH box filter
//                  (src/hella/src/convolution.cu:40-53: an xw x yw kernel of
//                  one value, anchor {xw/2, yw/2}, replicate border).
//
// The reference calls the forms without a stream context, which CUDA 13's
// NPP no longer has; the _Ctx forms take the context built below (device
// properties of the current device, the caller's stream).  Pointers are
// device pointers; steps are in bytes.  Returns the NppStatus (0 = success).
// Nothing in the product links this file.
#include <cuda_runtime.h>
#include <npp.h>

namespace {

int make_ctx(void *stream, NppStreamContext *ctx) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1000;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return -1001;
  ctx->hStream = (cudaStream_t)stream;
  ctx->nCudaDeviceId = dev;
  ctx->nMultiProcessorCount = prop.multiProcessorCount;
  ctx->nMaxThreadsPerMultiProcessor = prop.maxThreadsPerMultiProcessor;
  ctx->nMaxThreadsPerBlock = prop.maxThreadsPerBlock;
  ctx->nSharedMemPerBlock = prop.sharedMemPerBlock;
  ctx->nCudaDevAttrComputeCapabilityMajor = prop.major;
  ctx->nCudaDevAttrComputeCapabilityMinor = prop.minor;
  unsigned flags = 0;
  if (cudaStreamGetFlags((cudaStream_t)stream, &flags) != cudaSuccess) return -1002;
  ctx->nStreamFlags = flags;
  return 0;
}

}  // namespace

extern "C" int nr_filter_f32(const float *src, int src_step, int width, int height, float *dst, int dst_step,
                             const float *d_kernel, int kw, int kh, int ax, int ay, void *stream) {
  NppStreamContext ctx;
  int e = make_ctx(stream, &ctx);
  if (e) return e;
  const NppiSize size = {width, height};
  const NppiPoint off = {0, 0};
  return (int)nppiFilterBorder_32f_C1R_Ctx(src, src_step, size, off, dst, dst_step, size, d_kernel, NppiSize{kw, kh},
                                           NppiPoint{ax, ay}, NPP_BORDER_REPLICATE, ctx);
}

extern "C" int nr_filter_f16(const void *src, int src_step, int width, int height, void *dst, int dst_step,
                             const float *d_kernel, int kw, int kh, int ax, int ay, void *stream) {
  NppStreamContext ctx;
  int e = make_ctx(stream, &ctx);
  if (e) return e;
  const NppiSize size = {width, height};
  const NppiPoint off = {0, 0};
  return (int)nppiFilterBorder32f_16f_C1R_Ctx(static_cast<const Npp16f *>(src), src_step, size, off,
                                              static_cast<Npp16f *>(dst), dst_step, size, d_kernel,
                                              NppiSize{kw, kh}, NppiPoint{ax, ay}, NPP_BORDER_REPLICATE, ctx);
}
