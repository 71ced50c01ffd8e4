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
// Staging.  A work item is (beam, tile of DPT trials, 4S samples); the
// block walks the tables' channels CC at a time.  Host-built tile tables
// give, per (tile, channel), the smallest delay of the tile's trials (the
// first trial's, for an ascending DM list), the delay spread across the
// tile and the per-trial byte offsets, so every stage is
// one contiguous bulk copy per channel (the packed words [t0 + delay,
// + S + spread), two copies where the ring wraps) plus one for the offsets.
// Stage g of a block is issued by warp g mod 8 (lane i copies channel i)
// with cp.async.bulk (TMA) onto the full mbarrier of buffer g mod nbuf
// (2-4 buffers); every warp arrives on the buffer's empty mbarrier once it
// has summed the stage, which frees the buffer for stage g + nbuf.  No
// block-wide barrier sits in the loop.  Every wait is bounded: a wait that
// runs out sets bit 0 of the status word, drains the copies in flight
// (bounded again) and ends the block.
//
// Persistence.  The grid is sized to the resident blocks of the GPU and
// strides over the work items of every beam of the launch; items of one
// beam run in groups of `group` DM tiles per time tile, so that blocks
// resident together read overlapping windows of the ring through L2.
#include "hg_internal.h"
#include "hg_ptx.h"

#include <algorithm>
#include <type_traits>

namespace hg {
namespace {

constexpr int S = kPackS;
constexpr size_t kSmemBudget = 110 * 1024;  // two resident blocks per SM

__host__ __device__ constexpr int row_words(int max_spread) {
  // sh + S + spread words (sh < 4) rounded up to 16-byte chunks
  return ((S + max_spread + 6) + 3) / 4 * 4;
}
__host__ __device__ constexpr int off_width(int dpt) { return dpt < 4 ? 4 : dpt; }
constexpr int kMaxBuf = 4;        // staging buffers (pipeline depth)
constexpr int kBarBytes = 448;    // full[4] | empty[4] mbarriers | per warp: its staging cursor

// Words of one staging buffer: sh [cc] | off [cc][offw] | rows [cc][rowstride];
// every part is a multiple of 16 bytes.
__host__ __device__ constexpr int buf_words(int dpt, int cc, int rowstride) {
  return cc + cc * off_width(dpt) + cc * rowstride;
}
size_t smem_bytes(int dpt, int cc, int rowstride, int nbuf) {
  return kBarBytes + (size_t)nbuf * buf_words(dpt, cc, rowstride) * 4;
}

// Where one work item reads and writes.
struct Item {
  const uint32_t *packed;
  float *out;
  const int4 *meta;   // tile row of the tables
  const int *off;
  long w0;            // ring position of the item's first sample
  int t0, tile, dm_count;
  int nact;           // channels of the item's tables
};

// Beam of a work item (binary search over the beams' item prefixes).
__device__ __forceinline__ int beam_of(const DedispArgs &a, int item) {
  int lo = 0, hi = a.nbeam - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.beams[mid].item0 <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Channels summed for a work item.
__device__ __forceinline__ int item_nact(const DedispArgs &a, int item) {
  if (!a.beams) return a.nact;
  const DedispBeam &bm = a.beams[beam_of(a, item)];
  return bm.meta ? bm.nact : a.nact;
}

// VAR: the beam's own tables when it has them (else the launch's).
template <int DPT, bool VAR = false>
__device__ __forceinline__ Item item_at(const DedispArgs &a, int item) {
  const DedispBeam bm = a.beams ? a.beams[beam_of(a, item)] : a.one;
  const int ntiles = (bm.dm_count + DPT - 1) / DPT;
  const int l = item - bm.item0;
  const int per_group = a.group * a.ntt;
  const int g = l / per_group, r = l - g * per_group;
  const int gsz = min(a.group, ntiles - g * a.group);
  const int tt = r / gsz;
  Item it;
  it.tile = g * a.group + (r - tt * gsz);
  it.t0 = tt * 4 * S;
  it.w0 = (bm.win0 + it.t0) % a.R;
  it.packed = bm.packed;
  it.out = bm.out;
  it.dm_count = bm.dm_count;
  if constexpr (VAR) {
    const bool own = a.beams && bm.meta;
    it.nact = own ? bm.nact : a.nact;
    it.meta = (own ? bm.meta : a.tile_meta) + (size_t)it.tile * it.nact;
    it.off = (own ? bm.off : a.tile_off) + (size_t)it.tile * it.nact * off_width(DPT);
  } else {
    it.nact = a.nact;
    it.meta = a.tile_meta + (size_t)it.tile * a.nact;
    it.off = a.tile_off + (size_t)it.tile * a.nact * off_width(DPT);
  }
  return it;
}

// MODE picks how the integer adds are spread over the SM's pipes (the
// sums are identical): 0 = three-input adds throughout; 1 = load addresses
// as multiply-adds by a runtime 1 (FMA pipe); 2 = as 1, and the odd-sample
// lanes accumulated by multiply-adds as well; 3 = two-input address adds
// (which issue on the full-rate FMA pipes), odd lanes by multiply-adds.
// Byte permutes and three-input adds share the half-rate ALU pipe, and
// multiply-adds the half-rate heavy FMA pipe, so MODE 3 leaves 2.5 ALU
// and 2 multiply-add instructions per word.
//
// VAR: the launch's items differ in their number of stages (beams with
// tables of their own), so each warp walks a cursor over the items; else
// every item has ceil(a.nact / CC) stages and stage g maps to item and
// stage by division.
template <int DPT, int CC, int MODE, bool VAR>
__global__ void __launch_bounds__(kDedispThreads, 2) k_dedisp(DedispArgs a, int rowstride, int nbuf) {
  extern __shared__ __align__(128) uint32_t smem[];
  constexpr int OFFW = off_width(DPT);
  constexpr int NWARP = kDedispThreads / 32;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t bw4 = (uint32_t)buf_words(DPT, CC, rowstride) * 4u;
  const uint32_t rs4 = (uint32_t)rowstride * 4u;
  auto full_of = [&](int b) { return sbase + 8u * b; };
  auto empty_of = [&](int b) { return sbase + 32u + 8u * b; };
  auto sh_of = [&](int b) { return sbase + kBarBytes + (uint32_t)b * bw4; };
  auto off_of = [&](int b) { return sh_of(b) + CC * 4u; };
  auto rows_of = [&](int b) { return off_of(b) + CC * OFFW * 4u; };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t unit = (uint32_t)a.unit;  // 1, unknown to the compiler
  // Stage g of the block (the block's stages counted over its items in
  // order; an item has ceil(nact / CC) of them, nact its beam's channels)
  // is staged by warp g % 8, lane i copying channel i.  The item a warp is
  // staging (VAR: with a cursor to its next stage) is kept in shared memory
  // to spare registers.
  struct StagedFix {
    const uint32_t *packed;
    const int4 *meta;
    const int *off;
    long w0;
  };
  struct StagedVar {
    const uint32_t *packed;
    const int4 *meta;
    const int *off;
    long w0;
    int k, st, nst, nact;  // stage st of the nst stages of block-local item k
  };
  using Staged = std::conditional_t<VAR, StagedVar, StagedFix>;
  static_assert(64 + NWARP * sizeof(Staged) <= kBarBytes, "staging cursors");
  Staged *staged = reinterpret_cast<Staged *>(reinterpret_cast<char *>(smem) + 64 + sizeof(Staged) * warp);

  if (tid == 0) {
    for (int b = 0; b < nbuf; ++b) {
      mbar_init(full_of(b), 32);      // every lane of the staging warp arrives once per fill
      mbar_init(empty_of(b), NWARP);  // one arrival per warp once it is done reading
    }
    mbar_fence_init();
  }
  __syncthreads();
  if (blockIdx.x >= a.nitems) return;

  // lane 0: block-local item k into *staged (false past the block's items)
  auto load_item = [&](int k) -> bool {
    const int item = blockIdx.x + k * gridDim.x;
    if (item >= a.nitems) return false;
    const Item it = item_at<DPT, VAR>(a, item);
    if constexpr (VAR)
      *staged = Staged{it.packed, it.meta, it.off, it.w0, k, 0, (it.nact + CC - 1) / CC, it.nact};
    else
      *staged = Staged{it.packed, it.meta, it.off, it.w0};
    return true;
  };
  // lane 0: the cursor n stages on, over items without channels (false past
  // the block's last stage)
  auto advance = [&](int n) -> bool {
    if constexpr (VAR) {
      int st = staged->st + n;
      while (st >= staged->nst) {
        st -= staged->nst;
        if (!load_item(staged->k + 1)) return false;
      }
      staged->st = st;
    }
    return true;
  };
  const int nstage_u = (a.nact + CC - 1) / CC;  // !VAR: stages of every item
  const unsigned g_end =                        // !VAR: stages of the block
      VAR ? 0u : (unsigned)((a.nitems - 1 - blockIdx.x) / gridDim.x + 1) * (unsigned)nstage_u;
  unsigned g_next = (unsigned)warp;  // next stage this warp stages
  int staged_k = -1;                 // !VAR: block-local item held in *staged
  bool p_done;                       // no stage left for this warp
  if constexpr (VAR) {
    int more = 0;
    if (lane == 0) more = load_item(0) && advance(warp);
    p_done = !__shfl_sync(0xffffffffu, more, 0);
    __syncwarp();
  } else {
    p_done = false;  // unused: g_end bounds the stages
  }

  // Stages stage g_next into buffer g_next % nbuf; `block`: may wait for
  // the buffer to be released, else returns false if it is not free yet.
  auto issue = [&](bool block, bool *timed_out) -> bool {
    const unsigned g = g_next;
    const int b = (int)(g % (unsigned)nbuf);
    if (g >= (unsigned)nbuf) {
      const uint32_t par = ((g / nbuf) - 1u) & 1u;
      if (block) {
        if (!mbar_wait(empty_of(b), par)) {
          *timed_out = true;
          return false;
        }
      } else if (!mbar_test(empty_of(b), par)) {
        return false;
      }
    }
    int st;
    if constexpr (VAR) {
      st = staged->st;
    } else {
      const int k = (int)(g / (unsigned)nstage_u);
      st = (int)(g % (unsigned)nstage_u);
      if (k != staged_k) {
        if (lane == 0) load_item(k);
        staged_k = k;
        __syncwarp();
      }
    }
    int nact_st;
    if constexpr (VAR) nact_st = staged->nact;
    else nact_st = a.nact;
    const int k0 = st * CC, nc = min(CC, nact_st - k0);
    const uint32_t bar = full_of(b);
    fence_proxy_async();
    if (lane < nc) {
      const int4 mc = __ldg(staged->meta + k0 + lane);  // {channel, base delay, spread, 0}
      long p = staged->w0 + mc.y;
      while (p >= a.R) p -= a.R;
      const long a4 = p & ~3L;
      const int sh = (int)(p - a4);
      const int n16 = (sh + S + mc.z + 3) >> 2;  // 16-byte chunks, <= rowstride / 4
      sts32(sh_of(b) + lane * 4u, sh);
      const uint32_t obytes = lane == 0 ? (uint32_t)(nc * OFFW * 4) : 0u;
      mbar_arrive_tx(bar, (uint32_t)n16 * 16u + obytes);
      const uint32_t *src = staged->packed + (size_t)mc.x * a.R;
      uint32_t dst = rows_of(b) + (uint32_t)lane * rs4;
      long pos = a4;
      int left = n16;
      while (left > 0) {  // the ring may wrap inside the staged window
        const int n = (int)min((long)left, (a.R - pos) >> 2);
        bulk_g2s(dst, src + pos, (uint32_t)n * 16u, bar);
        dst += (uint32_t)n * 16u;
        left -= n;
        pos = 0;
      }
      if (lane == 0) bulk_g2s(off_of(b), staged->off + (size_t)k0 * OFFW, obytes, bar);
    } else {
      mbar_arrive(bar);
    }
    __syncwarp();
    g_next += NWARP;
    if constexpr (VAR) {
      int more = 0;
      if (lane == 0) more = advance(NWARP);
      p_done = !__shfl_sync(0xffffffffu, more, 0);
      __syncwarp();
    }
    return true;
  };
  // After a wait ran out: record it, let this warp's copies land, end.
  auto fail = [&](unsigned gs_c) {
    if (lane == 0 && a.err) atomicOr(a.err, 1);
    for (unsigned g = gs_c; g < g_next; ++g)
      if (g % NWARP == (unsigned)warp) mbar_wait(full_of((int)(g % nbuf)), (g / nbuf) & 1u);
  };

  unsigned gs_c = 0;  // stages consumed
  for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
    const int nact = VAR ? item_nact(a, item) : a.nact;
    const int nstage = VAR ? (nact + CC - 1) / CC : nstage_u;
    uint32_t acc_e[DPT], acc_o[DPT], tot[DPT][4];
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      acc_e[m] = acc_o[m] = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) tot[m][k] = 0u;
    }
    for (int st = 0; st < nstage; ++st) {
      {
        // keep up to nbuf stages in flight; the stage about to be read must be issued
        bool to = false;
        while ((VAR ? !p_done : g_next < g_end) && g_next < gs_c + nbuf)
          if (!issue(g_next <= gs_c, &to)) break;
        if (to) return fail(gs_c);
      }
      const int b = (int)(gs_c % (unsigned)nbuf), nc = min(CC, nact - st * CC);
      if (!mbar_wait(full_of(b), (gs_c / nbuf) & 1u)) return fail(gs_c);
      const uint32_t rbase = rows_of(b) + (uint32_t)tid * 4u;
      const uint32_t shb = sh_of(b), offb = off_of(b);
      // offsets are byte offsets (host-scaled): each load address is one add
      auto add_pair = [&](int ci) {
        const uint32_t r1 = rbase + (uint32_t)ci * rs4 + lds32(shb + ci * 4u) * 4u;
        const uint32_t r2 = rbase + (uint32_t)(ci + 1) * rs4 + lds32(shb + ci * 4u + 4u) * 4u;
#pragma unroll
        for (int q = 0; q < OFFW / 4; ++q) {
          const int4 x1 = lds128(offb + (uint32_t)(ci * OFFW + 4 * q) * 4u);
          const int4 x2 = lds128(offb + (uint32_t)((ci + 1) * OFFW + 4 * q) * 4u);
          const int o1[4] = {x1.x, x1.y, x1.z, x1.w}, o2[4] = {x2.x, x2.y, x2.z, x2.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int m = 4 * q + j;
            if (m < DPT) {
              constexpr bool kMadAddr = MODE == 1 || MODE == 2;
              const uint32_t w1 = lds32(kMadAddr ? (uint32_t)o1[j] * unit + r1 : r1 + (uint32_t)o1[j]);
              const uint32_t w2 = lds32(kMadAddr ? (uint32_t)o2[j] * unit + r2 : r2 + (uint32_t)o2[j]);
              acc_e[m] += __byte_perm(w1, 0u, 0x4240) + __byte_perm(w2, 0u, 0x4240);
              if (MODE >= 2) {
                acc_o[m] = __byte_perm(w1, 0u, 0x4341) * unit + acc_o[m];
                acc_o[m] = __byte_perm(w2, 0u, 0x4341) * unit + acc_o[m];
              } else {
                acc_o[m] += __byte_perm(w1, 0u, 0x4341) + __byte_perm(w2, 0u, 0x4341);
              }
            }
          }
        }
      };
      auto add_one = [&](int ci) {
        const uint32_t r1 = rbase + (uint32_t)ci * rs4 + lds32(shb + ci * 4u) * 4u;
#pragma unroll
        for (int q = 0; q < OFFW / 4; ++q) {
          const int4 x1 = lds128(offb + (uint32_t)(ci * OFFW + 4 * q) * 4u);
          const int o1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int m = 4 * q + j;
            if (m < DPT) {
              const uint32_t w1 = lds32(r1 + (uint32_t)o1[j]);
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
      __syncwarp();
      if (lane == 0) mbar_arrive(empty_of(b));  // this warp is done with buffer b
      ++gs_c;
      if ((st + 1) % (256 / CC) == 0) {  // 256 channels per 16-bit lane, then widen
#pragma unroll
        for (int m = 0; m < DPT; ++m) {
          tot[m][0] += acc_e[m] & 0xffffu;
          tot[m][2] += acc_e[m] >> 16;
          tot[m][1] += acc_o[m] & 0xffffu;
          tot[m][3] += acc_o[m] >> 16;
          acc_e[m] = acc_o[m] = 0u;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      tot[m][0] += acc_e[m] & 0xffffu;
      tot[m][2] += acc_e[m] >> 16;
      tot[m][1] += acc_o[m] & 0xffffu;
      tot[m][3] += acc_o[m] >> 16;
    }
    const Item it = item_at<DPT>(a, item);
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      const int i = it.tile * DPT + m;
      if (i >= it.dm_count) break;
      float *o = it.out + (size_t)i * a.out_stride;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int t = it.t0 + tid + k * S;
        if (t < a.nout) o[t] = (float)tot[m][k];
      }
    }
  }
}

// Block (x, job): tiles x, x + gridDim.x, ... of job `job`; a thread per
// channel of the job copies its table entry and dpt offsets.
__global__ void k_gather_tables(const int4 *__restrict__ meta, const int *__restrict__ off, int nch, int dpt,
                                const TableJob *__restrict__ jobs, const int *__restrict__ chans,
                                int4 *__restrict__ bmeta, int *__restrict__ boff) {
  const TableJob j = jobs[blockIdx.y];
  for (int tile = blockIdx.x; tile < j.ntiles; tile += gridDim.x)
    for (int k = threadIdx.x; k < j.nact; k += blockDim.x) {
      const size_t src = (size_t)tile * nch + chans[j.chans0 + k];
      const size_t dst = (size_t)j.meta0 + (size_t)tile * j.nact + k;
      bmeta[dst] = meta[src];
      for (int m = 0; m < dpt; ++m) boff[dst * dpt + m] = off[src * dpt + m];
    }
}

__global__ void k_pack(const uint8_t *__restrict__ plain, uint32_t *__restrict__ packed,
                       int nchan, long R, long q0, long nq, const uint8_t *__restrict__ keep,
                       const GulpPos *dpos) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  if (dpos) q0 = ((dpos->wpos - 3L * S) % R + R) % R;
  const size_t bc = (size_t)blockIdx.z * nchan + blockIdx.y;
  const size_t row = bc * (size_t)R;
  const long q = (q0 + i) % R;
  if (keep && !keep[bc]) {
    packed[row + q] = 0u;
    return;
  }
  const uint8_t *p = plain + row;
  const uint32_t b0 = p[q], b1 = p[(q + S) % R], b2 = p[(q + 2 * S) % R],
                 b3 = p[(q + 3 * S) % R];
  packed[row + q] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
}

// k_pack for 4-word-aligned ranges: thread i builds words q..q+3
// (q = q0 + 4i) from one 32-bit load at each of q, q+S, q+2S, q+3S and a
// 4x4 byte transpose, and stores them as one 16-byte word.  R % 4 == 0 and
// q0 % 4 == 0 keep every load and store aligned and no group straddles the
// ring's end.
__global__ void k_pack4(const uint8_t *__restrict__ plain, uint32_t *__restrict__ packed,
                        int nchan, long R, long q0, long ngroups, const uint8_t *__restrict__ keep,
                        const GulpPos *dpos) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ngroups) return;
  if (dpos) q0 = ((dpos->wpos - 3L * S) % R + R) % R;
  const size_t bc = (size_t)blockIdx.z * nchan + blockIdx.y;
  const size_t row = bc * (size_t)R;
  long q = q0 + 4 * i;
  while (q >= R) q -= R;
  uint4 *dst = reinterpret_cast<uint4 *>(packed + row + q);
  if (keep && !keep[bc]) {
    *dst = make_uint4(0u, 0u, 0u, 0u);
    return;
  }
  uint32_t a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    long pos = q + (long)k * S;
    while (pos >= R) pos -= R;
    a[k] = *reinterpret_cast<const uint32_t *>(plain + row + pos);  // byte j = sample pos + j
  }
  const uint32_t t0 = __byte_perm(a[0], a[1], 0x5140), t1 = __byte_perm(a[2], a[3], 0x5140);
  const uint32_t t2 = __byte_perm(a[0], a[1], 0x7362), t3 = __byte_perm(a[2], a[3], 0x7362);
  *dst = make_uint4(__byte_perm(t0, t1, 0x5410), __byte_perm(t0, t1, 0x7632), __byte_perm(t2, t3, 0x5410),
                    __byte_perm(t2, t3, 0x7632));
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


// ---------------------------------------------------------------------
// Add mode 4: sub-band sums shared by the trials of a tile.
//
// Within a tile of kSubDPT trials, a group of kSubG adjacent active
// channels c0..c3 contributes x[c0][t+d0] + x[c1][t+d1] + x[c2][t+d2] +
// x[c3][t+d3] to trial d (dk = delay(ck, d)).  The relative delays
// dk - d0 take few distinct values over the tile's trials (3.7 "patterns"
// per 16 trials and 4 channels on the full beam's DM list), so a stage
// stages the group's four rows (as the 8-channel stages do), the block
// builds one row of four-channel sums per pattern in shared memory (16-bit
// lanes, <= 4 x 255, two words per packed position: samples k = 0,2 and
// k = 1,3), and each trial adds the row of its pattern at its offset: one
// 8-byte shared load and two adds per trial and group, against four loads,
// eight byte permutes and two three-input adds channel by channel.  The
// sums are integers, so any grouping gives the same totals.
//
// Host tables per (tile, group): a record of ints
//   [npat, pattern words, channels in the group, 0,
//    toff[16]   byte offset of trial m's read in the pattern rows (+ 8 j),
//    per pattern: L (words), row offset (words), 0, 0, o0, o1, o2, o3]
// where pattern p's row holds L words (256 plus the spread of its trials'
// head delays) and its word q sums staged word sh_k + o_k + q of each
// channel k.  Pattern rows are built with one block barrier per stage,
// into two alternating buffers, so a stage's sums and the next stage's
// building never touch the same buffer.
constexpr int kSubRecHdr = 20;  // ints before the patterns: header + toff[16]

__device__ __forceinline__ void sts64(uint32_t addr, uint32_t x, uint32_t y) {
  asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(addr), "r"(x), "r"(y) : "memory");
}
__device__ __forceinline__ uint2 lds64(uint32_t addr) {
  uint2 v;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(addr));
  return v;
}
__device__ __forceinline__ void sts128(uint32_t addr, int4 v) {
  asm volatile("st.shared.v4.s32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

__host__ __device__ constexpr uint32_t sub_buf_bytes(int rowstride, int recb) {
  return 16u + (uint32_t)recb + (uint32_t)kSubG * (uint32_t)rowstride * 4u;
}
__host__ __device__ constexpr uint32_t sub_pat_bytes(int words) {
  return 64u + (uint32_t)((words + 1) / 2 * 2) * 8u;  // 16-byte multiple: the next buffer's header is read as int4
}

__global__ void __launch_bounds__(kDedispThreads, 2)
    k_dedisp_sub(DedispArgs a, int rowstride, int nbuf, int recb, int pwords) {
  extern __shared__ __align__(128) uint32_t smem[];
  constexpr int NWARP = kDedispThreads / 32;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t rs4 = (uint32_t)rowstride * 4u;
  const uint32_t bufb = sub_buf_bytes(rowstride, recb);
  const uint32_t patb = sub_pat_bytes(pwords);
  auto full_of = [&](int b) { return sbase + 8u * b; };
  auto empty_of = [&](int b) { return sbase + 32u + 8u * b; };
  const uint32_t abort_at = sbase + 64u;
  auto sh_of = [&](int b) { return sbase + kBarBytes + (uint32_t)b * bufb; };
  auto rec_of = [&](int b) { return sh_of(b) + 16u; };
  auto rows_of = [&](int b) { return rec_of(b) + (uint32_t)recb; };
  auto pat_of = [&](unsigned g) { return sbase + kBarBytes + (uint32_t)nbuf * bufb + (g & 1u) * patb; };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  struct Staged {  // the item a warp is staging, kept in shared memory to spare registers
    const uint32_t *packed;
    const int4 *meta;
    long w0;
    int tile, pad;
  };
  static_assert(128 + NWARP * sizeof(Staged) <= kBarBytes, "staging cursors");
  Staged *staged = reinterpret_cast<Staged *>(reinterpret_cast<char *>(smem) + 128 + sizeof(Staged) * warp);

  if (tid == 0) {
    for (int b = 0; b < nbuf; ++b) {
      mbar_init(full_of(b), 32);
      mbar_init(empty_of(b), NWARP);
    }
    sts32(abort_at, 0);
    mbar_fence_init();
  }
  __syncthreads();
  if (blockIdx.x >= a.nitems) return;

  const int ngroups = (a.nact + kSubG - 1) / kSubG;
  const unsigned g_end = (unsigned)((a.nitems - 1 - blockIdx.x) / gridDim.x + 1) * (unsigned)ngroups;
  unsigned g_next = (unsigned)warp;  // next stage this warp stages
  int staged_k = -1;

  // Stages stage g_next (group g_next % ngroups of the block's item
  // g_next / ngroups) into buffer g_next % nbuf.
  auto issue = [&](bool block, bool *timed_out) -> bool {
    const unsigned g = g_next;
    const int b = (int)(g % (unsigned)nbuf);
    if (g >= (unsigned)nbuf) {
      const uint32_t par = ((g / nbuf) - 1u) & 1u;
      if (block) {
        if (!mbar_wait(empty_of(b), par)) {
          *timed_out = true;
          return false;
        }
      } else if (!mbar_test(empty_of(b), par)) {
        return false;
      }
    }
    const int k = (int)(g / (unsigned)ngroups), st = (int)(g % (unsigned)ngroups);
    if (k != staged_k) {
      if (lane == 0) {
        const Item it = item_at<kSubDPT>(a, blockIdx.x + k * gridDim.x);
        *staged = Staged{it.packed, it.meta, it.w0, it.tile, 0};
      }
      staged_k = k;
      __syncwarp();
    }
    const int k0 = st * kSubG, nc = min(kSubG, a.nact - k0);
    const uint32_t bar = full_of(b);
    fence_proxy_async();
    if (lane < nc) {
      const int4 mc = __ldg(staged->meta + k0 + lane);  // {channel, base delay, spread, 0}
      long p = staged->w0 + mc.y;
      while (p >= a.R) p -= a.R;
      const long a4 = p & ~3L;
      const int sh = (int)(p - a4);
      const int n16 = (sh + S + mc.z + 3) >> 2;  // 16-byte chunks, <= rowstride / 4
      sts32(sh_of(b) + lane * 4u, sh);
      int2 ix = make_int2(0, 0);
      if (lane == 0) ix = __ldg(a.sub_index + (size_t)staged->tile * ngroups + st);  // {pool int, bytes}
      mbar_arrive_tx(bar, (uint32_t)n16 * 16u + (uint32_t)ix.y);
      const uint32_t *src = staged->packed + (size_t)mc.x * a.R;
      uint32_t dst = rows_of(b) + (uint32_t)lane * rs4;
      long pos = a4;
      int left = n16;
      while (left > 0) {  // the ring may wrap inside the staged window
        const int n = (int)min((long)left, (a.R - pos) >> 2);
        bulk_g2s(dst, src + pos, (uint32_t)n * 16u, bar);
        dst += (uint32_t)n * 16u;
        left -= n;
        pos = 0;
      }
      if (lane == 0) bulk_g2s(rec_of(b), a.sub_pool + ix.x, (uint32_t)ix.y, bar);
    } else {
      mbar_arrive(bar);
    }
    __syncwarp();
    g_next += NWARP;
    return true;
  };

  unsigned gs_c = 0;  // stages consumed
  for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
    uint32_t acc_e[kSubDPT], acc_o[kSubDPT], tot[kSubDPT][4];
#pragma unroll
    for (int m = 0; m < kSubDPT; ++m) {
      acc_e[m] = acc_o[m] = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) tot[m][k] = 0u;
    }
    for (int st = 0; st < ngroups; ++st) {
      bool bad = false;
      {
        bool to = false;
        while (g_next < g_end && g_next < gs_c + nbuf)
          if (!issue(g_next <= gs_c, &to)) break;
        bad = to;
      }
      const int b = (int)(gs_c % (unsigned)nbuf);
      if (!bad && !mbar_wait(full_of(b), (gs_c / nbuf) & 1u)) bad = true;
      const uint32_t pb = pat_of(gs_c);
      if (!bad) {
        // ---- build the stage's pattern rows (flattened: word w of the rows to thread w % 256)
        const uint32_t rb = rec_of(b);
        const int4 hd = lds128(rb);  // npat, words, channels, 0
        if (tid < 4) sts128(pb + 16u * tid, lds128(rb + 16u + 16u * tid));  // toff[16] for the sums
        const uint32_t r0 = rows_of(b);
        const int gc = hd.z;
        uint32_t shk[kSubG];
#pragma unroll
        for (int k = 0; k < kSubG; ++k) shk[k] = k < gc ? lds32(sh_of(b) + 4u * k) : 0u;
        for (int p = 0; p < hd.x; ++p) {
          const int4 pa = lds128(rb + 4u * (kSubRecHdr + 8 * p));      // L, row offset
          const int4 po = lds128(rb + 4u * (kSubRecHdr + 8 * p + 4));  // o0..o3
          int q = (tid - pa.y) & (S - 1);
          if (q >= pa.x) continue;
          uint32_t dst = pb + 64u + 8u * (uint32_t)(pa.y + q);
          uint32_t ra = r0 + 4u * (shk[0] + po.x + q);
          uint32_t rbw = r0 + rs4 + 4u * (shk[1] + po.y + q);
          uint32_t rc = r0 + 2u * rs4 + 4u * (shk[2] + po.z + q);
          uint32_t rd = r0 + 3u * rs4 + 4u * (shk[3] + po.w + q);
          if (gc == kSubG) {
            for (; q < pa.x; q += S) {
              const uint32_t w0 = lds32(ra), w1 = lds32(rbw), w2 = lds32(rc), w3 = lds32(rd);
              const uint32_t e = __byte_perm(w0, 0u, 0x4240) + __byte_perm(w1, 0u, 0x4240) +
                                 (__byte_perm(w2, 0u, 0x4240) + __byte_perm(w3, 0u, 0x4240));
              const uint32_t o = __byte_perm(w0, 0u, 0x4341) + __byte_perm(w1, 0u, 0x4341) +
                                 (__byte_perm(w2, 0u, 0x4341) + __byte_perm(w3, 0u, 0x4341));
              sts64(dst, e, o);
              dst += 8u * S;
              ra += 4u * S;
              rbw += 4u * S;
              rc += 4u * S;
              rd += 4u * S;
            }
          } else {  // the last group of a channel list that is not a multiple of four
            for (; q < pa.x; q += S) {
              uint32_t e = 0u, o = 0u;
              const uint32_t w0 = lds32(ra);
              e += __byte_perm(w0, 0u, 0x4240);
              o += __byte_perm(w0, 0u, 0x4341);
              if (gc > 1) {
                const uint32_t w1 = lds32(rbw);
                e += __byte_perm(w1, 0u, 0x4240);
                o += __byte_perm(w1, 0u, 0x4341);
              }
              if (gc > 2) {
                const uint32_t w2 = lds32(rc);
                e += __byte_perm(w2, 0u, 0x4240);
                o += __byte_perm(w2, 0u, 0x4341);
              }
              sts64(dst, e, o);
              dst += 8u * S;
              ra += 4u * S;
              rbw += 4u * S;
              rc += 4u * S;
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(empty_of(b));  // this warp is done with the staged rows of buffer b
        if (bad) {
          if (a.err) atomicOr(a.err, 1);
          sts32(abort_at, 1);
        }
      }
      __syncthreads();  // the stage's pattern rows are complete (and the previous stage's sums done)
      if (lds32(abort_at)) {
        // a wait ran out somewhere in the block: let this warp's copies land, end
        for (unsigned g = gs_c; g < g_next; ++g)
          if (g % NWARP == (unsigned)warp) mbar_wait(full_of((int)(g % nbuf)), (g / nbuf) & 1u);
        return;
      }
      // ---- sums: each trial adds its pattern row at its offset
      const uint32_t rows = pb + 64u + 8u * (uint32_t)tid;
#pragma unroll
      for (int q4 = 0; q4 < kSubDPT / 4; ++q4) {
        const int4 to = lds128(pb + 16u * q4);
        const int t4[4] = {to.x, to.y, to.z, to.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint2 v = lds64(rows + (uint32_t)t4[j]);
          acc_e[4 * q4 + j] += v.x;
          acc_o[4 * q4 + j] += v.y;
        }
      }
      ++gs_c;
      if ((st + 1) % (256 / kSubG) == 0) {  // 64 groups of <= 1020 per 16-bit lane, then widen
#pragma unroll
        for (int m = 0; m < kSubDPT; ++m) {
          tot[m][0] += acc_e[m] & 0xffffu;
          tot[m][2] += acc_e[m] >> 16;
          tot[m][1] += acc_o[m] & 0xffffu;
          tot[m][3] += acc_o[m] >> 16;
          acc_e[m] = acc_o[m] = 0u;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < kSubDPT; ++m) {
      tot[m][0] += acc_e[m] & 0xffffu;
      tot[m][2] += acc_e[m] >> 16;
      tot[m][1] += acc_o[m] & 0xffffu;
      tot[m][3] += acc_o[m] >> 16;
    }
    const Item it = item_at<kSubDPT>(a, item);
#pragma unroll
    for (int m = 0; m < kSubDPT; ++m) {
      const int i = it.tile * kSubDPT + m;
      if (i >= it.dm_count) break;
      float *o = it.out + (size_t)i * a.out_stride;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int t = it.t0 + tid + k * S;
        if (t < a.nout) o[t] = (float)tot[m][k];
      }
    }
  }
}

}  // namespace

// Smallest and largest delay of channel c over trials d0..d1 (the first
// and the last for an ascending DM list).
static void tile_delay_range(const int *delays, int nchan, int c, int d0, int d1, int *lo, int *hi) {
  *lo = *hi = delays[(size_t)d0 * nchan + c];
  for (int d = d0 + 1; d <= d1; ++d) {
    const int v = delays[(size_t)d * nchan + c];
    *lo = std::min(*lo, v);
    *hi = std::max(*hi, v);
  }
}

int dedisp_spread(const int *delays, int nchan, const int *chans, int nact, int dm_first,
                  int dm_count, int dpt) {
  const int dlast = dm_first + dm_count - 1;
  int spread = 0;
  for (int d0 = dm_first; d0 <= dlast; d0 += dpt) {
    const int d1 = std::min(d0 + dpt - 1, dlast);
    for (int k = 0; k < nact; ++k) {
      int lo, hi;
      tile_delay_range(delays, nchan, chans[k], d0, d1, &lo, &hi);
      spread = std::max(spread, hi - lo);
    }
  }
  return spread;
}

// Staging buffers for a tile shape: the deepest pipeline (up to kMaxBuf)
// that fits the budget of two resident blocks per SM; 0 if even two do not.
int dedisp_nbuf(int dpt, int cc, int max_spread) {
  for (int nb = kMaxBuf; nb >= 2; --nb)
    if (smem_bytes(dpt, cc, row_words(max_spread), nb) <= kSmemBudget) return nb;
  return 0;
}

size_t dedisp_smem_bytes(int dpt, int cc, int max_spread) {
  const int nb = dedisp_nbuf(dpt, cc, max_spread);
  return nb ? smem_bytes(dpt, cc, row_words(max_spread), nb) : 0;
}

DedispTables dedisp_tables(const int *delays, int nchan, const int *chans, int nact, int dm_first,
                           int dm_count, int dpt, int cc) {
  DedispTables t;
  const int dlast = dm_first + dm_count - 1;
  if (dpt > 0) {
    t.dpt = dpt;
    t.max_spread = dedisp_spread(delays, nchan, chans, nact, dm_first, dm_count, dpt);
  } else {
    for (int d : {16, 8, 4, 2, 1}) {
      const int spread = dedisp_spread(delays, nchan, chans, nact, dm_first, dm_count, d);
      if (dedisp_smem_bytes(d, cc, spread) || d == 1) {
        t.dpt = d;
        t.max_spread = spread;
        break;
      }
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
      int base, top;
      tile_delay_range(delays, nchan, c, d0, d1, &base, &top);
      t.meta[(size_t)i * nact + k] = make_int4(c, base, top - base, 0);
      int *o = &t.off[((size_t)i * nact + k) * t.offw];
      for (int m = 0; m < t.dpt; ++m)  // byte offsets into the staged row
        o[m] = 4 * (delays[(size_t)std::min(d0 + m, dlast) * nchan + c] - base);
    }
  }
  return t;
}

// ---- add mode 4 tables (see k_dedisp_sub)
SubTables dedisp_sub_tables(const int *delays, int nchan, const int *chans, int nact, int dm_first,
                            int dm_count) {
  SubTables t;
  const int dlast = dm_first + dm_count - 1;
  t.ntiles = (dm_count + kSubDPT - 1) / kSubDPT;
  t.ngroups = (nact + kSubG - 1) / kSubG;
  t.meta.resize((size_t)t.ntiles * nact);
  t.index.resize((size_t)t.ntiles * t.ngroups);
  std::vector<int> base(nact), rel(kSubDPT * kSubG), h(kSubDPT), pid(kSubDPT);
  for (int i = 0; i < t.ntiles; ++i) {
    const int d0 = dm_first + i * kSubDPT, d1 = std::min(d0 + kSubDPT - 1, dlast), nt = d1 - d0 + 1;
    for (int k = 0; k < nact; ++k) {
      int lo, hi;
      tile_delay_range(delays, nchan, chans[k], d0, d1, &lo, &hi);
      t.meta[(size_t)i * nact + k] = make_int4(chans[k], lo, hi - lo, 0);
      base[k] = lo;
      t.max_spread = std::max(t.max_spread, hi - lo);
    }
    for (int g = 0; g < t.ngroups; ++g) {
      const int k0 = g * kSubG, gc = std::min(kSubG, nact - k0);
      auto dl = [&](int m, int k) { return delays[(size_t)(d0 + m) * nchan + chans[k0 + k]]; };
      // patterns: the relative delays of the group's channels, in order of first use
      std::vector<int> first;  // trial that defines each pattern
      for (int m = 0; m < nt; ++m) {
        for (int k = 0; k < gc; ++k) rel[m * kSubG + k] = dl(m, k) - dl(m, 0);
        h[m] = dl(m, 0) - base[k0];
        int p = 0;
        for (; p < (int)first.size(); ++p)
          if (std::equal(&rel[m * kSubG], &rel[m * kSubG] + gc, &rel[first[p] * kSubG])) break;
        if (p == (int)first.size()) first.push_back(m);
        pid[m] = p;
      }
      const int npat = (int)first.size();
      std::vector<int> rec(kSubRecHdr + 8 * npat, 0);
      int words = 0;
      for (int p = 0; p < npat; ++p) {
        int qlo = 1 << 30, qhi = -1;
        for (int m = 0; m < nt; ++m)
          if (pid[m] == p) {
            qlo = std::min(qlo, h[m]);
            qhi = std::max(qhi, h[m]);
          }
        int *pr = &rec[kSubRecHdr + 8 * p];
        pr[0] = S + qhi - qlo;  // L
        pr[1] = words;          // row offset
        for (int k = 0; k < gc; ++k)
          pr[4 + k] = base[k0] + qlo + rel[first[p] * kSubG + k] - base[k0 + k];  // >= 0, see the kernel
        for (int m = 0; m < nt; ++m)
          if (pid[m] == p) rec[4 + m] = 8 * (words + h[m] - qlo);
        words += pr[0];
      }
      rec[0] = npat;
      rec[1] = words;
      rec[2] = gc;
      t.index[(size_t)i * t.ngroups + g] = make_int2((int)t.pool.size(), (int)(rec.size() * 4));
      t.pool.insert(t.pool.end(), rec.begin(), rec.end());
      t.max_words = std::max(t.max_words, words);
      t.max_rec = std::max(t.max_rec, (int)(rec.size() * 4));
    }
  }
  return t;
}

// Shared memory of the add-mode-4 kernel with `nbuf` staging buffers.
size_t dedisp_sub_smem(int max_spread, int max_words, int max_rec, int nbuf) {
  return kBarBytes + (size_t)nbuf * sub_buf_bytes(row_words(max_spread), max_rec) +
         2 * (size_t)sub_pat_bytes(max_words);
}

namespace {

template <int DPT, int CC, int MODE, bool VAR>
cudaError_t launch_var(const DedispArgs &a, cudaStream_t s) {
  const int rowstride = row_words(a.max_spread);
  int nbuf = a.nbuf ? a.nbuf : dedisp_nbuf(DPT, CC, a.max_spread);
  if (!nbuf) nbuf = 2;  // very coarse DM lists: one block per SM
  if (nbuf < 2 || nbuf > kMaxBuf) return cudaErrorInvalidValue;
  const size_t smem = smem_bytes(DPT, CC, rowstride, nbuf);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  auto kern = k_dedisp<DPT, CC, MODE, VAR>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kDedispThreads, smem)) != cudaSuccess)
    return e;
  const int grid = std::max(1, std::min(a.nitems, std::max(1, per_sm) * sms));
  kern<<<grid, kDedispThreads, smem, s>>>(a, rowstride, nbuf);
  count_launches(1);
  return cudaGetLastError();
}

// Items with differing stage counts come only from tables of 8 or more
// trials per tile.
template <int DPT, int CC, int MODE>
cudaError_t launch(const DedispArgs &a, cudaStream_t s) {
  if constexpr (DPT >= 8) {
    if (a.varied) return launch_var<DPT, CC, MODE, true>(a, s);
  } else {
    if (a.varied) return cudaErrorInvalidValue;
  }
  return launch_var<DPT, CC, MODE, false>(a, s);
}

template <int DPT>
cudaError_t launch_cc(const DedispArgs &a, cudaStream_t s) {
  if (DPT < 8 && a.mode != 0) return cudaErrorInvalidValue;  // modes 1-3: 8 and 16-trial tiles
  switch (a.cc * 4 + (DPT < 8 ? 0 : a.mode)) {
    case 32: return launch<DPT, 8, 0>(a, s);
    case 64: return launch<DPT, 16, 0>(a, s);
    case 33: return launch<DPT, 8, DPT < 8 ? 0 : 1>(a, s);
    case 65: return launch<DPT, 16, DPT < 8 ? 0 : 1>(a, s);
    case 34: return launch<DPT, 8, DPT < 8 ? 0 : 2>(a, s);
    case 66: return launch<DPT, 16, DPT < 8 ? 0 : 2>(a, s);
    case 35: return launch<DPT, 8, DPT < 8 ? 0 : 3>(a, s);
    case 67: return launch<DPT, 16, DPT < 8 ? 0 : 3>(a, s);
  }
  return cudaErrorInvalidValue;
}

// Add mode 4: staging depth 3 (2 if 3 does not fit) within the two-blocks
// budget, else the deepest that fits one block per SM.
cudaError_t launch_sub(const DedispArgs &a, cudaStream_t s) {
  if (a.dpt != kSubDPT || a.varied || !a.sub_index || !a.sub_pool || a.sub_words < S || a.sub_rec < 16 ||
      a.sub_rec % 16 != 0)
    return cudaErrorInvalidValue;
  const int rowstride = row_words(a.max_spread);
  int nbuf = a.nbuf;
  if (!nbuf) {
    nbuf = 2;
    for (int nb = 3; nb >= 2; --nb)
      if (dedisp_sub_smem(a.max_spread, a.sub_words, a.sub_rec, nb) <= kSmemBudget) {
        nbuf = nb;
        break;
      }
  }
  if (nbuf < 2 || nbuf > kMaxBuf) return cudaErrorInvalidValue;
  const size_t smem = dedisp_sub_smem(a.max_spread, a.sub_words, a.sub_rec, nbuf);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_dedisp_sub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dedisp_sub, kDedispThreads, smem)) !=
      cudaSuccess)
    return e;
  const int grid = std::max(1, std::min(a.nitems, std::max(1, per_sm) * sms));
  k_dedisp_sub<<<grid, kDedispThreads, smem, s>>>(a, rowstride, nbuf, a.sub_rec, a.sub_words);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t dedisperse(const DedispArgs &a, cudaStream_t s) {
  if (a.nitems <= 0 || a.nout <= 0 || a.nact <= 0) return cudaSuccess;
  if (a.R % 4 != 0 || a.ntt <= 0 || a.group <= 0 || a.nbeam <= 0) return cudaErrorInvalidValue;
  if (a.varied && !a.beams) return cudaErrorInvalidValue;
  if (a.mode == 4) return launch_sub(a, s);
  if (a.mode == 5 || a.mode == 6) return dedisperse_pairs(a, s);
  switch (a.dpt) {
    case 16: return launch_cc<16>(a, s);
    case 8: return launch_cc<8>(a, s);
    case 4: return launch_cc<4>(a, s);
    case 2: return launch_cc<2>(a, s);
    case 1: return launch_cc<1>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t gather_tables(const int4 *meta, const int *off, int nch, int dpt, const TableJob *jobs, int njobs,
                          int max_tiles, const int *chans, int4 *bmeta, int *boff, cudaStream_t s) {
  if (njobs <= 0 || max_tiles <= 0) return cudaSuccess;
  if (dpt < 8 || njobs > 65535) return cudaErrorInvalidValue;
  k_gather_tables<<<dim3((unsigned)std::min(max_tiles, 64), (unsigned)njobs), 256, 0, s>>>(meta, off, nch, dpt,
                                                                                         jobs, chans, bmeta, boff);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t pack_ring(const uint8_t *plain, uint32_t *packed, int nbeam, int nchan,
                      long R, long q0, long nq, cudaStream_t s, const uint8_t *keep) {
  if (nq <= 0) return cudaSuccess;
  q0 = ((q0 % R) + R) % R;
  nq = std::min(nq, R);  // each ring position once
  if (R % 4 == 0 && q0 % 4 == 0 && nq % 4 == 0) {
    const dim3 grid((unsigned)((nq / 4 + 255) / 256), nchan, nbeam);
    k_pack4<<<grid, 256, 0, s>>>(plain, packed, nchan, R, q0, nq / 4, keep, nullptr);
    count_launches(1);
    return cudaGetLastError();
  }
  const dim3 grid((unsigned)((nq + 255) / 256), nchan, nbeam);
  k_pack<<<grid, 256, 0, s>>>(plain, packed, nchan, R, q0, nq, keep, nullptr);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t pack_gulp_dev(const uint8_t *plain, uint32_t *packed, int nbeam, int nchan, long R,
                          int gulp, const GulpPos *pos, cudaStream_t s, const uint8_t *keep) {
  const long nq = std::min((long)gulp + 3L * S, R);  // each ring position once
  if (R % 4 == 0 && gulp % 4 == 0 && nq % 4 == 0) {  // wpos is then a multiple of 4 as well
    const dim3 grid((unsigned)((nq / 4 + 255) / 256), nchan, nbeam);
    k_pack4<<<grid, 256, 0, s>>>(plain, packed, nchan, R, 0, nq / 4, keep, pos);
    count_launches(1);
    return cudaGetLastError();
  }
  const dim3 grid((unsigned)((nq + 255) / 256), nchan, nbeam);
  k_pack<<<grid, 256, 0, s>>>(plain, packed, nchan, R, 0, nq, keep, pos);
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

// Shared-memory reads: every thread reads 16 bytes a load, a warp 512
// consecutive bytes (no bank conflicts), from a 32 KiB block buffer, at an
// address that moves with the iteration.  The loads are volatile, so none
// is merged with another or moved out of the loop, and their values are
// folded into the stored result.
__global__ void __launch_bounds__(256) k_smem_read_peak(unsigned *out, int iters) {
  __shared__ __align__(16) uint32_t buf[8192];
  for (int i = threadIdx.x; i < 8192; i += blockDim.x) buf[i] = i * 2654435761u;
  __syncthreads();
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(buf);
  uint32_t acc = 0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t w = ((threadIdx.x + (uint32_t)k * 256u + (uint32_t)i * 32u) & 2047u) * 16u;
      int4 v;
      asm volatile("ld.volatile.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
                   : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                   : "r"(base + w));
      acc += (uint32_t)(v.x ^ v.y) + (uint32_t)(v.z ^ v.w);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
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

extern "C" hella_status hella_smem_read_peak(int device, double *bytes_per_s) {
  if (!bytes_per_s) return HELLA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return HELLA_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 6, threads = 256, iters = 2048;
  unsigned *out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, (size_t)blocks * threads * 4) != cudaSuccess) return HELLA_ERR_ALLOC;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    hg::k_smem_read_peak<<<blocks, threads>>>(out, iters);
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
  *bytes_per_s = (double)blocks * threads * iters * 8 * 16 / (best * 1e-3);
  return st;
}
