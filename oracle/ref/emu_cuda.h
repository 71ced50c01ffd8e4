/*
 * emu_cuda.h -- just enough CUDA to run the reference's flagger,
 * statistics, smoothing and peak-finding sources on the CPU, so that their
 * outputs can pin the oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Kernels become host functions executed once per (block, thread); blocks
 * whose kernels synchronise run their threads as cooperative fibers, so
 * __syncthreads and __shfl_down_sync behave as on a GPU.  fp16 arithmetic
 * comes from CUDA's own cuda_fp16.h host implementation.  The CUDA runtime
 * calls the sources make are served from host memory (emu_cuda.cpp).
 * Force-included ahead of every reference translation unit.
 */
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <unistd.h> /* nvcc's host include chain provides it */

#include <cstdint>
#include <functional>

#undef __global__
#define __global__
#undef __shared__
#define __shared__ static

/* The kernel built-ins, as globals the launcher sets (host code that names
 * a local gridDim/blockDim simply shadows them, as under nvcc). */
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

namespace emu {
void syncthreads();
uint64_t exchange(uint64_t v, unsigned src_lane_offset);
void launch(dim3 grid, dim3 block, bool cooperative, const std::function<void()> &body);
}  // namespace emu

#ifndef warpSize
#define warpSize 32
#endif

inline void __syncthreads() { emu::syncthreads(); }

template <typename T>
T __shfl_down_sync(unsigned, T v, unsigned delta, int = 32) {
  static_assert(sizeof(T) <= 8, "shuffle of a wide type");
  uint64_t bits = 0;
  __builtin_memcpy(&bits, &v, sizeof(T));
  bits = emu::exchange(bits, delta);
  T r;
  __builtin_memcpy(&r, &bits, sizeof(T));
  return r;
}

/* NPP filters the reference calls whose non-_Ctx forms CUDA 13 dropped. */
#include <nppdefs.h>
extern "C" NppStatus nppiFilterBorder32f_16f_C1R(const Npp16f *pSrc, Npp32s nSrcStep, NppiSize oSrcSize,
                                                 NppiPoint oSrcOffset, Npp16f *pDst, Npp32s nDstStep,
                                                 NppiSize oSizeROI, const Npp32f *pKernel, NppiSize oKernelSize,
                                                 NppiPoint oAnchor, NppiBorderType eBorderType);
extern "C" NppStatus nppiFilterBorder_32f_C1R(const Npp32f *pSrc, Npp32s nSrcStep, NppiSize oSrcSize,
                                              NppiPoint oSrcOffset, Npp32f *pDst, Npp32s nDstStep,
                                              NppiSize oSizeROI, const Npp32f *pKernel, NppiSize oKernelSize,
                                              NppiPoint oAnchor, NppiBorderType eBorderType);
