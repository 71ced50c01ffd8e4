// noalloc.cu -- hdd_execute_noalloc (include/hella_dedisp.h): dedispersion
// for callers that cannot allocate device memory while they run.
//
// Its scratch (dedispersion tile tables, channel-major staging copy and
// packed ring) is carved out of one file-scope device array instead of
// cudaMalloc'd buffers.  Host code never uses the array's name as an
// address: that name is only a host-side stand-in for the symbol.  The
// device address is looked up once per device with cudaGetSymbolAddress
// (with that device current) and handed to the kernels.
#include "hella_dedisp.h"
#include "hg_internal.h"
#include "hg_plan.h"

#include <mutex>

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[HDD_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current);
// the first call per device resolves it and clears the status word (the
// first 256 bytes), which later calls only read and clear after reporting.
hdd_error scratch_for(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return HDD_INVALID_DEVICE_INDEX;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return HDD_INTERNAL_GPU_ERROR;
    }
    if (cudaMemset(p, 0, 256) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
      cudaGetLastError();
      return HDD_INTERNAL_GPU_ERROR;
    }
    g_scratch_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_scratch_addr[device]);
  return HDD_NO_ERROR;
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace

extern "C" hdd_error hdd_execute_noalloc(hdd_plan plan, hdd_size nsamps, const hdd_byte *in,
                                         hdd_size in_nbits, hdd_size in_stride, hdd_byte *out,
                                         hdd_size out_nbits, hdd_size out_stride, unsigned flags) {
  if (!plan) return HDD_INVALID_PLAN;
  if (!in || !out) return HDD_INVALID_POINTER;
  const hg::PlanView v = hg::plan_view(plan);
  if (v.ndms == 0) return HDD_NO_DM_LIST_SET;
  if (flags & HDD_HOST_POINTERS) return HDD_INVALID_FLAG_COMBINATION;  // device pointers only
  if ((flags & HDD_WAIT) && (flags & HDD_ASYNC)) return HDD_INVALID_FLAG_COMBINATION;
  if (in_nbits != 8) return HDD_UNSUPPORTED_IN_NBITS;
  if (out_nbits != 32) return HDD_UNSUPPORTED_OUT_NBITS;
  if (nsamps <= (hdd_size)v.max_delay) return HDD_TOO_FEW_NSAMPS;
  if (nsamps > (hdd_size)(65535u * 32u)) return HDD_UNKNOWN_ERROR;  // transpose grid limit, as hdd_execute_guru
  const int nout = (int)(nsamps - v.max_delay);
  if (in_stride < (hdd_size)v.nchans) return HDD_INVALID_STRIDE;
  if (out_stride % 4 != 0 || out_stride < (hdd_size)nout * 4) return HDD_INVALID_STRIDE;

  // scratch layout: status | tile meta | tile offsets | staging [nchans][R] | packed [nchans][R]
  // (the tile tables are built on the host once per plan and DM range)
  const hg::DedispTables &tb = hg::plan_host_tables(plan, 0, v.ndms);
  const long R = ((long)nsamps + 3) / 4 * 4;
  const size_t o_err = 0;
  const size_t o_meta = 256;
  const size_t o_off = o_meta + align256(tb.meta.size() * sizeof(int4));
  const size_t o_plain = o_off + align256(tb.off.size() * sizeof(int));
  const size_t o_packed = o_plain + align256((size_t)v.nchans * R);
  const size_t total = o_packed + (size_t)v.nchans * R * 4;
  if (total > HDD_NOALLOC_SCRATCH_BYTES) return HDD_STATIC_SCRATCH_EXCEEDED;

  if (cudaSetDevice(v.device) != cudaSuccess) return HDD_INVALID_DEVICE_INDEX;
  if (cudaPeekAtLastError() != cudaSuccess) return HDD_PRIOR_GPU_ERROR;
  unsigned char *base = nullptr;
  hdd_error e = scratch_for(v.device, &base);
  if (e != HDD_NO_ERROR) return e;
  cudaStream_t s = (cudaStream_t)v.stream;
  int4 *d_meta = reinterpret_cast<int4 *>(base + o_meta);
  int *d_off = reinterpret_cast<int *>(base + o_off);
  uint8_t *d_plain = base + o_plain;
  uint32_t *d_packed = reinterpret_cast<uint32_t *>(base + o_packed);
  int *d_err = reinterpret_cast<int *>(base + o_err);

  // The tables, staging copy and packed ring are rewritten by every call.
  // The status word is not: a staging timeout sets it and it stays set until
  // a synchronous call reads it, reports it and clears it, so a timeout in an
  // HDD_ASYNC call surfaces at the next synchronous call.
  if (!tb.meta.empty() &&
      (cudaMemcpyAsync(d_meta, tb.meta.data(), tb.meta.size() * sizeof(int4), cudaMemcpyHostToDevice, s) !=
           cudaSuccess ||
       cudaMemcpyAsync(d_off, tb.off.data(), tb.off.size() * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess))
    return HDD_MEM_COPY_FAILED;
  if (hg::transpose_tf(in, in_stride, (int)nsamps, v.nchans, d_plain, R, s) != cudaSuccess)
    return HDD_INTERNAL_GPU_ERROR;
  if (hg::pack_ring(d_plain, d_packed, 1, v.nchans, R, 0, R, s) != cudaSuccess)
    return HDD_INTERNAL_GPU_ERROR;
  float *dout = reinterpret_cast<float *>(out);
  if (v.nact == 0) {
    for (int d = 0; d < v.ndms; ++d)
      if (cudaMemsetAsync(out + (size_t)d * out_stride, 0, (size_t)nout * 4, s) != cudaSuccess)
        return HDD_INTERNAL_GPU_ERROR;
  } else {
    hg::DeviceTables dt{d_meta, d_off, tb.dpt, tb.max_spread, v.nact, 8};
    const hg::DedispArgs a =
        hg::single_beam_args(dt, d_packed, R, 0, 0, v.ndms, nout, dout, (long)(out_stride / 4), d_err);
    if (hg::dedisperse(a, s) != cudaSuccess) return HDD_INTERNAL_GPU_ERROR;
  }
  if (!(flags & HDD_ASYNC)) {
    if (cudaStreamSynchronize(s) != cudaSuccess) return HDD_INTERNAL_GPU_ERROR;
    int err = 0;
    if (cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return HDD_INTERNAL_GPU_ERROR;
    if (err) {  // a staging wait of this call or of an earlier HDD_ASYNC call timed out
      if (cudaMemsetAsync(d_err, 0, sizeof(int), s) != cudaSuccess) return HDD_INTERNAL_GPU_ERROR;
      return HDD_INTERNAL_GPU_ERROR;
    }
  }
  return HDD_NO_ERROR;
}
