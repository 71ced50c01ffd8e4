// pairs.cu -- add modes 5 and 6 of the dedispersion: rows of channel
// groups, pairs (g = 2) or quads (g = 4) (hg_internal.h).
//
// Same exact integer sums as k_dedisp (out[d][t] = sum over active channels
// c of x[c][t + delay(c, d)], the operation casm-hella obtains from
// dedisp_execute_adv, src/hella/src/dedisperse.cpp:17-48), computed in two
// launches per window:
//
// k_pair_build: one block per (group, 4096 window positions for pairs, 2048
//   for quads).  The group's channels' packed words of the chunk (for
//   channel i widened by the group's range of relative delays r_i) are read
//   from the ring once into shared memory as 16-bit lanes (bytes 0 and 2 of
//   a packed word are the samples p and p + 512), eight loads in flight per
//   thread, then one warp per row writes every row of the group from them:
//   row(r)[p] = x[c0][p] + sum_i x[c_i][p + r_i], the next row's metadata
//   loaded while a row is written.  Reads are the ring once per group;
//   writes the rows, coalesced, with streaming stores.  A row keeps, tile
//   by tile, only the words its trials read where those span less than a
//   1024-sample tile.
//
// k_pair_sum: the persistent staging pipeline of k_dedisp (work item =
//   16-trial tile x 1024 output samples, stages issued warp by warp with
//   cp.async.bulk onto full/empty mbarriers, every wait bounded) over stage
//   records instead of channels.  A stage stages the windows of the rows
//   its groups use (lane i copies row i) and the record's trial offsets;
//   thread j then reads, per group and trial, the words j and j + 256 of
//   the trial's window: four output samples (j, j+256, j+512, j+768) in two
//   SWAR registers of 16-bit lanes, two groups per three-input add.  The
//   lanes are widened into 32-bit totals every pair_lanecap(g) groups.
//
// Per group and trial the inner loop is two shared loads and one add for
// 4g channel-samples, against two loads, four byte permutes and two adds
// per eight in k_dedisp; shared-memory traffic is 2/g bytes per
// channel-sample, so the sums are bound by shared-memory bandwidth, and
// the build by its row writes (g = 4: about three times the rows of g = 2).
#include "hg_internal.h"
#include "hg_ptx.h"

#include <algorithm>
#include <array>
#include <cstring>

namespace hg {
namespace {

constexpr int S = kPackS;
constexpr int kTileSamples = 4 * S;
// window positions per build block: 4096 for pairs, 2048 for quads (whose
// four channel windows would otherwise leave three blocks per SM)
__host__ __device__ constexpr int build_chunk(int g) { return g <= 2 ? 4096 : 2048; }
constexpr int kBarHdr = 448;              // full[4] | empty[4] | per-warp staging cursors
constexpr size_t kSmemBudget = 113 * 1024;  // two resident blocks per SM (228 KB less 1 KB a block)
constexpr int kMaxBuf = 4;

__host__ __device__ constexpr int stage_hdr_bytes(int cc) { return 16 + cc * kPairDPT * 4; }

// Window positions a row spans from its first position: all its words for
// a single run, (ntt - 1) tiles of 1024 and one stride for tiled rows.
__device__ __forceinline__ long row_positions(const DedispArgs &a, int r) {
  const int stride = a.pair_rtile[r];
  return stride == kTileSamples ? (long)a.pair_rwords[r] : (long)(a.ntt - 1) * kTileSamples + stride;
}

// A row's metadata, all of it loaded together (one wait per row).
struct BuildRow {
  int w, z1, z2, z3, stride, words;
  long long off;
};

__device__ __forceinline__ BuildRow build_row(const DedispArgs &a, int r, bool quad) {
  const int4 in = a.pair_rinfo[r];
  const int4 in2 = quad ? a.pair_rinfo2[r] : make_int4(-1, -1, 0, 0);
  return BuildRow{in.w, in.z, in2.z, in2.w, a.pair_rtile[r], a.pair_rwords[r], a.pair_roff[r]};
}

template <int G>
__global__ void __launch_bounds__(256, G == 4 ? 5 : 6) k_pair_build(DedispArgs a) {
  extern __shared__ uint32_t sm[];
  constexpr int kBuildCH = build_chunk(G);
  const int k = blockIdx.y, z = blockIdx.z;  // group, beam of the launch
  const long P0 = (long)blockIdx.x * kBuildCH;
  const DedispBeam bm = a.beams ? a.beams[z] : a.one;
  const int r0 = a.pair_prow[k];
  const int r1 = a.pair_rend ? a.pair_rend[(size_t)z * a.pair_npair + k] : a.pair_prow[k + 1];
  // the group's channels and relative-delay ranges, loaded beside the chunk test's rows
  const int4 i0 = a.pair_rinfo[r0], j0 = a.pair_rinfo2[r0];
  int2 rr[kPairGMax];
  rr[0] = make_int2(0, 0);
#pragma unroll
  for (int i = 1; i < kPairGMax; ++i) rr[i] = i < G ? a.pair_prange[k * (kPairGMax - 1) + i - 1] : make_int2(0, 0);
  int any = 0;  // does a row of the group cover a position of this chunk?
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int w = a.pair_rinfo[r].w;
    any |= P0 < (long)w + row_positions(a, r) && P0 + kBuildCH > (long)w;
  }
  if (!__syncthreads_or(any)) return;
  const int ch[kPairGMax] = {i0.x, i0.y, G == 4 ? j0.x : -1, G == 4 ? j0.y : -1};  // -1: fewer channels
  const long R = a.R;
  // channel i's words for positions [P0 + rmin_i, P0 + kBuildCH + rmax_i) at sm + off[i];
  // window position p lies at ring word (win0 + p) mod R
  int off[kPairGMax + 1], rmin[kPairGMax];
  long base[kPairGMax];
  int nwin = 0;
#pragma unroll
  for (int i = 0; i < kPairGMax; ++i) {
    off[i] = nwin;
    rmin[i] = rr[i].x;
    base[i] = 0;
    if (i >= G || ch[i] < 0) continue;
    long b = (bm.win0 + P0 + rr[i].x) % R;
    base[i] = b < 0 ? b + R : b;
    nwin += kBuildCH + rr[i].y - rr[i].x;
  }
  off[kPairGMax] = nwin;
  // all the group's windows as one run of words, kLoads ring loads in flight per thread (a
  // window word's channel: the last i with off[i] <= q; absent channels hold no words)
  constexpr int kLoads = 8;
  for (int q0 = threadIdx.x; q0 < nwin; q0 += kLoads * blockDim.x) {
    uint32_t v[kLoads];
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < nwin) {
        int i = 0;
#pragma unroll
        for (int j = 1; j < G; ++j) i += q >= off[j] ? 1 : 0;
        const int c = i == 0 ? ch[0] : i == 1 ? ch[1] : i == 2 ? ch[2] : ch[3];
        const long b = i == 0 ? base[0] : i == 1 ? base[1] : i == 2 ? base[2] : base[3];
        const int o = i == 0 ? off[0] : i == 1 ? off[1] : i == 2 ? off[2] : off[3];
        long pos = b + (q - o);
        if (pos >= R) pos %= R;
        v[u] = bm.packed[(size_t)c * R + pos];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < nwin) sm[q] = __byte_perm(v[u], 0u, 0x4240);
    }
  }
  __syncthreads();
  // one warp per row: the row's metadata is loaded once for 2048-4096 words, the next row's
  // while this one is written
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  int r = r0 + (threadIdx.x >> 5);
  BuildRow nx{};
  if (r < r1) nx = build_row(a, r, G == 4);
  for (; r < r1; r += nwarp) {
    const BuildRow in = nx;
    if (r + nwarp < r1) nx = build_row(a, r + nwarp, G == 4);
    const long npos = in.stride == kTileSamples ? (long)in.words : (long)(a.ntt - 1) * kTileSamples + in.stride;
    if (P0 >= (long)in.w + npos || P0 + kBuildCH <= (long)in.w) continue;
    uint32_t *dst = a.pair_rows + (size_t)z * a.pair_rows_stride + in.off;
    // word q of the chunk, q = p - P0, of channel i for this row's r_i
    const int s1 = off[1] + in.z1 - rmin[1], s2 = off[2] + in.z2 - rmin[2], s3 = off[3] + in.z3 - rmin[3];
    // the row's tiles: tile tt holds positions [first + 1024 tt, + stride) at words tt * stride on
    // (one run from word 0 when stride = 1024)
    const int stride = in.stride;
    const long rel0 = P0 - in.w;  // chunk start relative to the row's first position
    const int tt0 = (int)max(0L, rel0 / kTileSamples - 1);
    const int tt1 = (int)min((long)a.ntt - 1, (rel0 + kBuildCH) / kTileSamples);
    for (int tt = stride == kTileSamples ? 0 : tt0; tt <= (stride == kTileSamples ? 0 : tt1); ++tt) {
      // positions of this tile's words (the whole row for stride 1024), clipped to the chunk
      const long pb = (long)in.w + (long)tt * kTileSamples;
      const long pe = stride == kTileSamples ? (long)in.w + in.words : pb + stride;
      const long lo = max(P0, pb), hi = min(P0 + kBuildCH, pe);
      if (lo >= hi) continue;
      const int first = (int)(lo - P0), last = (int)(hi - P0);
      const long d0l = (long)tt * stride + (P0 - pb);  // word of chunk offset q is d0 + q
      uint32_t *dt = dst + d0l;
      // rows are read back by other blocks much later: streaming stores
      if (G == 4 && ch[3] >= 0) {
        for (int q = first + lane; q < last; q += 32) __stcs(dt + q, sm[q] + sm[s1 + q] + sm[s2 + q] + sm[s3 + q]);
      } else if (G == 4 && ch[2] >= 0) {
        for (int q = first + lane; q < last; q += 32) __stcs(dt + q, sm[q] + sm[s1 + q] + sm[s2 + q]);
      } else if (ch[1] >= 0) {
        for (int q = first + lane; q < last; q += 32) __stcs(dt + q, sm[q] + sm[s1 + q]);
      } else {
        for (int q = first + lane; q < last; q += 32) __stcs(dt + q, sm[q]);
      }
    }
  }
}

__device__ __forceinline__ void pair_item(const DedispArgs &a, int ntiles, int l, int *tile, int *tt) {
  const int per_group = a.group * a.ntt;
  const int g = l / per_group, r = l - g * per_group;
  const int gsz = min(a.group, ntiles - g * a.group);
  *tt = r / gsz;
  *tile = g * a.group + (r - *tt * gsz);
}

// MULTI: the launch serves several beams (a.beams, batched context): each
// item looks up its beam; else the one beam's record stays in registers.
template <int CC, bool MULTI>
__global__ void __launch_bounds__(kDedispThreads, 2) k_pair_sum(DedispArgs a, int bufbytes, int nbuf) {
  extern __shared__ __align__(128) uint32_t smem[];
  constexpr int DPT = kPairDPT;
  constexpr int NWARP = kDedispThreads / 32;
  constexpr int HB = stage_hdr_bytes(CC);
  const int REC = pair_rec_int4(CC);
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  auto full_of = [&](int b) { return sbase + 8u * b; };
  auto empty_of = [&](int b) { return sbase + 32u + 8u * b; };
  auto buf_of = [&](int b) { return sbase + kBarHdr + (uint32_t)b * (uint32_t)bufbytes; };
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the stage a warp stages next: stage st of the nst stages of block-local item k
  struct Cursor {
    int k, st, s0, nst, t0, z;  // z: beam of the item in the launch
  };
  static_assert(64 + NWARP * sizeof(Cursor) <= kBarHdr, "staging cursors");
  Cursor *cur = reinterpret_cast<Cursor *>(reinterpret_cast<char *>(smem) + 64) + warp;
  if (tid == 0) {
    for (int b = 0; b < nbuf; ++b) {
      mbar_init(full_of(b), 32);      // every lane of the staging warp arrives once per fill
      mbar_init(empty_of(b), NWARP);  // one arrival per warp once it is done reading
    }
    mbar_fence_init();
  }
  __syncthreads();
  if (blockIdx.x >= a.nitems) return;

  // Beam z of launch item `item` and the item's tile and time tile: the
  // items of the launch's beams follow one another (beam z's from
  // beams[z].item0 - beams[0].item0 on; a beam without trials has none).
  const DedispBeam b0 = MULTI ? a.one : (a.beams ? a.beams[0] : a.one);
  auto locate = [&](int item, int *z, int *tile, int *tt) -> DedispBeam {
    int zz = 0;
    DedispBeam bz = b0;
    if (MULTI) {
      const int g = a.beams[0].item0 + item;
      while (zz + 1 < a.nbeam && a.beams[zz + 1].item0 <= g) ++zz;
      bz = a.beams[zz];
      item = g - bz.item0;
    }
    *z = zz;
    pair_item(a, (bz.dm_count + DPT - 1) / DPT, item, tile, tt);
    return bz;
  };
  auto load_item = [&](int k) -> bool {  // lane 0
    const int item = blockIdx.x + k * gridDim.x;
    if (item >= a.nitems) return false;
    int z, tile, tt;
    locate(item, &z, &tile, &tt);
    const int s0 = a.pair_tile_st[tile];
    *cur = Cursor{k, 0, s0, a.pair_tile_st[tile + 1] - s0, tt * kTileSamples, z};
    return true;
  };
  auto advance = [&](int n) -> bool {  // lane 0
    int st = cur->st + n;
    while (st >= cur->nst) {
      st -= cur->nst;
      if (!load_item(cur->k + 1)) return false;
    }
    cur->st = st;
    return true;
  };
  unsigned g_next = (unsigned)warp;  // next stage this warp stages
  bool p_done;                       // no stage left for this warp
  {
    int more = 0;
    if (lane == 0) more = load_item(0) && advance(warp);
    p_done = !__shfl_sync(0xffffffffu, more, 0);
    __syncwarp();
  }
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
    const int4 *r = a.pair_rec + (size_t)(cur->s0 + cur->st) * REC;
    const int tt = cur->t0 / kTileSamples;
    const int nrows = __ldg(&r->y);
    const uint32_t bar = full_of(b);
    fence_proxy_async();
    if (lane < nrows) {
      // {first word (low, high), words | byte slot / 16 << 16, the row's words per time tile}
      const int4 rw = __ldg(r + 1 + CC * DPT / 4 + lane);
      const long start = (long)(((unsigned long long)(unsigned)rw.y << 32) | (unsigned)rw.x);
      const uint32_t nb = ((uint32_t)rw.z & 0xffffu) * 4u, slot = ((uint32_t)rw.z >> 16) * 16u;
      mbar_arrive_tx(bar, nb + (lane == 0 ? (uint32_t)HB : 0u));
      const uint32_t *rows = MULTI ? a.pair_rows + (size_t)cur->z * a.pair_rows_stride : a.pair_rows;
      bulk_g2s(buf_of(b) + HB + slot, rows + start + (long)tt * rw.w, nb, bar);
      if (lane == 0) bulk_g2s(buf_of(b), r, HB, bar);
    } else {
      mbar_arrive(bar);
    }
    __syncwarp();
    g_next += NWARP;
    int more = 0;
    if (lane == 0) more = advance(NWARP);
    p_done = !__shfl_sync(0xffffffffu, more, 0);
    __syncwarp();
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
    int z, tile, tt;
    const DedispBeam bm = locate(item, &z, &tile, &tt);
    const int nstage = a.pair_tile_st[tile + 1] - a.pair_tile_st[tile];
    uint32_t acc_a[DPT], acc_b[DPT], tot[DPT][4];  // acc_a: samples j, j+512; acc_b: j+256, j+768
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      acc_a[m] = acc_b[m] = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) tot[m][k] = 0u;
    }
    int npairs = 0;  // groups in the 16-bit lanes
    for (int st = 0; st < nstage; ++st) {
      {
        bool to = false;
        while (!p_done && g_next < gs_c + nbuf)
          if (!issue(g_next <= gs_c, &to)) break;
        if (to) return fail(gs_c);
      }
      const int b = (int)(gs_c % (unsigned)nbuf);
      if (!mbar_wait(full_of(b), (gs_c / nbuf) & 1u)) return fail(gs_c);
      const uint32_t hb = buf_of(b), ob = hb + 16u, rb = hb + (uint32_t)HB + (uint32_t)tid * 4u;
      const int ng = (int)lds32(hb);
      auto add2 = [&](int i) {  // pairs i and i + 1
#pragma unroll
        for (int q = 0; q < DPT / 4; ++q) {
          const int4 x1 = lds128(ob + (uint32_t)(i * DPT + 4 * q) * 4u);
          const int4 x2 = lds128(ob + (uint32_t)((i + 1) * DPT + 4 * q) * 4u);
          const int o1[4] = {x1.x, x1.y, x1.z, x1.w}, o2[4] = {x2.x, x2.y, x2.z, x2.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int m = 4 * q + j;
            const uint32_t p1 = rb + (uint32_t)o1[j], p2 = rb + (uint32_t)o2[j];
            acc_a[m] += lds32(p1) + lds32(p2);
            acc_b[m] += lds32(p1 + 4u * S) + lds32(p2 + 4u * S);
          }
        }
      };
      auto add1 = [&](int i) {
#pragma unroll
        for (int q = 0; q < DPT / 4; ++q) {
          const int4 x1 = lds128(ob + (uint32_t)(i * DPT + 4 * q) * 4u);
          const int o1[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int m = 4 * q + j;
            const uint32_t p1 = rb + (uint32_t)o1[j];
            acc_a[m] += lds32(p1);
            acc_b[m] += lds32(p1 + 4u * S);
          }
        }
      };
      if (ng == CC) {
#pragma unroll
        for (int i = 0; i < CC; i += 2) add2(i);
      } else {
        int i = 0;
        for (; i + 1 < ng; i += 2) add2(i);
        if (i < ng) add1(i);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(empty_of(b));  // this warp is done with buffer b
      ++gs_c;
      npairs += ng;
      if (npairs + CC > a.pair_lanecap) {
#pragma unroll
        for (int m = 0; m < DPT; ++m) {
          tot[m][0] += acc_a[m] & 0xffffu;
          tot[m][2] += acc_a[m] >> 16;
          tot[m][1] += acc_b[m] & 0xffffu;
          tot[m][3] += acc_b[m] >> 16;
          acc_a[m] = acc_b[m] = 0u;
        }
        npairs = 0;
      }
    }
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      tot[m][0] += acc_a[m] & 0xffffu;
      tot[m][2] += acc_a[m] >> 16;
      tot[m][1] += acc_b[m] & 0xffffu;
      tot[m][3] += acc_b[m] >> 16;
    }
    const int t0 = tt * kTileSamples;
#pragma unroll
    for (int m = 0; m < DPT; ++m) {
      const int i = tile * DPT + m;
      if (i >= bm.dm_count) break;
      float *o = bm.out + (size_t)i * a.out_stride;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int t = t0 + tid + k * S;
        if (t < a.nout) o[t] = (float)tot[m][k];
      }
    }
  }
}

template <int CC, bool MULTI>
cudaError_t launch_sum(const DedispArgs &a, cudaStream_t s) {
  const int bufbytes = stage_hdr_bytes(CC) + a.pair_stage;
  int nbuf = a.nbuf;
  if (!nbuf) {  // deepest pipeline within the two-blocks budget, else two buffers
    nbuf = 2;
    for (int nb = kMaxBuf; nb >= 2; --nb)
      if (kBarHdr + (size_t)nb * bufbytes <= kSmemBudget) {
        nbuf = nb;
        break;
      }
  }
  if (nbuf < 2 || nbuf > kMaxBuf) return cudaErrorInvalidValue;
  const size_t smem = kBarHdr + (size_t)nbuf * bufbytes;
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  auto kern = k_pair_sum<CC, MULTI>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kDedispThreads, smem)) != cudaSuccess)
    return e;
  const int grid = std::max(1, std::min(a.nitems, std::max(1, per_sm) * sms));
  kern<<<grid, kDedispThreads, smem, s>>>(a, bufbytes, nbuf);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

PairTables dedisp_pair_tables(const int *delays, int nchan, const int *chans, int nact, int dm_first,
                              int dm_count, int cc, int ntt, int g) {
  PairTables t;
  t.g = g;
  t.cc = cc;
  t.ntt = ntt;
  t.dm_count = dm_count;
  t.ntiles = (dm_count + kPairDPT - 1) / kPairDPT;
  t.npair = (nact + g - 1) / g;
  const int stage_max = pair_stage_budget(cc);
  auto dl = [&](int d, int c) { return delays[(size_t)(dm_first + d) * nchan + c]; };
  // rows: per group, one per distinct pattern (r_1, r_2, r_3) of relative
  // delays, in increasing (lexicographic) order
  using Pat = std::array<int, kPairGMax - 1>;
  std::vector<Pat> rel(dm_count), u;
  t.row_of.assign((size_t)dm_count * t.npair, 0);
  t.prow.assign(t.npair + 1, 0);
  t.prange.assign((size_t)t.npair * (kPairGMax - 1), make_int2(0, 0));
  for (int k = 0; k < t.npair; ++k) {
    int c[kPairGMax];
    for (int i = 0; i < kPairGMax; ++i) c[i] = i < g && g * k + i < nact ? chans[g * k + i] : -1;
    for (int d = 0; d < dm_count; ++d)
      for (int i = 1; i < kPairGMax; ++i) rel[d][i - 1] = c[i] >= 0 ? dl(d, c[i]) - dl(d, c[0]) : 0;
    u = rel;
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    const int base = (int)t.rinfo.size();
    for (const Pat &v : u) {
      t.rinfo.push_back(make_int4(c[0], c[1], v[0], 1 << 30));
      t.rinfo2.push_back(make_int4(c[2], c[3], v[1], v[2]));
    }
    for (int d = 0; d < dm_count; ++d) {
      const int id = base + (int)(std::lower_bound(u.begin(), u.end(), rel[d]) - u.begin());
      t.row_of[(size_t)d * t.npair + k] = id;
      t.rinfo[id].w = std::min(t.rinfo[id].w, dl(d, c[0]));
    }
    for (int i = 1; i < kPairGMax; ++i) {
      int lo = 0, hi = 0;
      for (size_t j = 0; j < u.size(); ++j) {
        lo = j ? std::min(lo, u[j][i - 1]) : u[j][i - 1];
        hi = j ? std::max(hi, u[j][i - 1]) : u[j][i - 1];
      }
      t.prange[(size_t)k * (kPairGMax - 1) + i - 1] = make_int2(lo, hi);
      t.max_span = std::max(t.max_span, hi - lo);
    }
    t.prow[k + 1] = (int)t.rinfo.size();
  }
  t.nrows = (int)t.rinfo.size();
  // per row, the union of its copies' windows within a time tile: [lo, hi) words from its first position
  std::vector<long long> lo(t.nrows, 1LL << 60), hi(t.nrows, 0);
  int max_nw = 0;
  // stage records
  const int REC = pair_rec_int4(cc);
  const int offs0 = 4, rows0 = 4 + cc * kPairDPT;  // int positions in a record
  std::vector<int> rec(REC * 4);
  struct Fix {
    size_t rec_int;  // int index of the row entry in t.rec
    int row, bal;
  };
  std::vector<Fix> fixes;
  std::vector<Fix> pending;
  int ng = 0, nr = 0, bytes = 0;
  auto flush = [&]() {
    const size_t at = t.rec.size() * 4;
    for (Fix f : pending) fixes.push_back(Fix{at + f.rec_int, f.row, f.bal});
    pending.clear();
    rec[0] = ng;
    rec[1] = nr;
    const size_t n0 = t.rec.size();
    t.rec.resize(n0 + REC);
    std::memcpy(&t.rec[n0], rec.data(), rec.size() * sizeof(int));
    t.max_stage = std::max(t.max_stage, bytes);
    std::fill(rec.begin(), rec.end(), 0);
    ng = nr = bytes = 0;
  };
  int ids[kPairDPT], av[kPairDPT];
  t.tile_st.push_back(0);
  for (int i = 0; i < t.ntiles; ++i) {
    const int d0 = i * kPairDPT, nt = std::min(kPairDPT, dm_count - d0);
    for (int k = 0; k < t.npair; ++k) {
      const int c0 = chans[g * k];
      int uid[kPairDPT], ub[kPairDPT], us[kPairDPT], nu = 0;
      for (int m = 0; m < nt; ++m) {
        ids[m] = t.row_of[(size_t)(d0 + m) * t.npair + k];
        av[m] = dl(d0 + m, c0) - t.rinfo[ids[m]].w;
        int j = 0;
        while (j < nu && uid[j] != ids[m]) ++j;
        if (j == nu) {
          uid[nu] = ids[m];
          ub[nu] = us[nu] = av[m];
          ++nu;
        } else {
          ub[j] = std::min(ub[j], av[m]);
          us[j] = std::max(us[j], av[m]);
        }
      }
      int add = 0, bal[kPairDPT], nw[kPairDPT];
      for (int j = 0; j < nu; ++j) {
        const int sh = ub[j] & 3;
        bal[j] = ub[j] - sh;
        nw[j] = (2 * S + (us[j] - ub[j]) + sh + 3) / 4 * 4;
        add += nw[j] * 4;
      }
      if (ng > 0 && (ng == cc || nr + nu > kPairRowsMax || bytes + add > stage_max)) flush();
      for (int j = 0; j < nu; ++j) {
        const int slot = bytes;
        for (int m = 0; m < nt; ++m)
          if (ids[m] == uid[j]) rec[offs0 + ng * kPairDPT + m] = slot + (av[m] - bal[j]) * 4;
        int *rw = &rec[rows0 + 4 * nr];
        rw[2] = (nw[j] & 0xffff) | (slot / 16) << 16;  // words (< 2^16) | byte slot / 16
        max_nw = std::max(max_nw, nw[j]);
        pending.push_back(Fix{(size_t)(rows0 + 4 * nr), uid[j], bal[j]});
        lo[uid[j]] = std::min(lo[uid[j]], (long long)bal[j]);
        hi[uid[j]] = std::max(hi[uid[j]], (long long)bal[j] + nw[j]);
        ++nr;
        bytes += nw[j] * 4;
      }
      ++ng;
    }
    if (ng > 0) flush();
    t.tile_st.push_back((int)(t.rec.size() / REC));
  }
  // Row layout.  A row keeps, for each time tile tt, the words its copies read: [tt * 1024 + lo,
  // tt * 1024 + hi) of its positions.  When hi - lo < 1024 the tiles' windows do not meet and are
  // stored one after another (tile stride hi - lo words); else the row is one run from lo (stride
  // 1024: the tiles' windows overlap).  Word i then holds position
  //   first + (i / stride) * 1024 + i % stride,   first = (smallest delay of its trials) + lo,
  // and a copy of tile tt starts at word tt * stride + (bal - lo).  Offsets and lengths stay
  // multiples of 4 words, so every copy starts 16-byte aligned.
  t.roff.resize(t.nrows);
  t.rwords.resize(t.nrows);
  t.rtile.resize(t.nrows);
  long long off = 0;
  for (int r = 0; r < t.nrows; ++r) {
    const long long span = hi[r] - lo[r];  // multiple of 4: lo and hi are
    const int stride = span < kTileSamples ? (int)span : kTileSamples;
    const long long w = (long long)(ntt - 1) * stride + span;
    t.rinfo[r].w += (int)lo[r];
    t.roff[r] = off;
    t.rwords[r] = (int)w;
    t.rtile[r] = stride;
    off += w;
    t.npos = std::max(t.npos, (long)t.rinfo[r].w + (long)(ntt - 1) * kTileSamples + (long)span);
  }
  t.words = (long)off;
  if (max_nw > 0xffff) t.max_stage = 1 << 30;  // a copy longer than its 16-bit field: no launch takes these
  int *ri = reinterpret_cast<int *>(t.rec.data());
  for (const Fix &f : fixes) {
    const unsigned long long start = (unsigned long long)(t.roff[f.row] + f.bal - lo[f.row]);
    ri[f.rec_int] = (int)(unsigned)(start & 0xffffffffull);
    ri[f.rec_int + 1] = (int)(unsigned)(start >> 32);
    ri[f.rec_int + 3] = t.rtile[f.row];
  }
  return t;
}

void pair_row_ends(const PairTables &t, int count, int *ends) {
  for (int k = 0; k < t.npair; ++k) {
    int e = t.prow[k];
    for (int d = 0; d < std::min(count, t.dm_count); ++d) e = std::max(e, t.row_of[(size_t)d * t.npair + k] + 1);
    ends[k] = e;
  }
}

cudaError_t dedisperse_pairs(const DedispArgs &a, cudaStream_t s) {
  const int g = a.pair_g;
  if ((a.beams && (a.nbeam < 1 || a.nbeam > kPairMaxBeams || (a.nbeam > 1 && a.pair_rows_stride <= 0))) ||
      a.dpt != kPairDPT || (a.mode != 5 && a.mode != 6) || (g != 2 && g != 4) ||
      !a.pair_rows || !a.pair_rec || !a.pair_tile_st || !a.pair_rinfo || !a.pair_rinfo2 || !a.pair_roff ||
      !a.pair_rwords || !a.pair_rtile || !a.pair_prow || !a.pair_prange || a.pair_npair <= 0 ||
      a.pair_npair > 65535 ||
      a.pair_stage <= 0 || a.pair_stage % 16 != 0 || a.pair_span < 0 || a.pair_lanecap < 1 ||
      a.pair_lanecap > pair_lanecap(g))
    return cudaErrorInvalidValue;
  if (a.R <= 0 || (!a.beams && a.one.win0 < 0)) return cudaErrorInvalidValue;
  // the group's channel windows: ch words for c0, ch + its r range for the others
  const int ch = build_chunk(g);
  const size_t bsmem = ((size_t)g * ch + (size_t)(g - 1) * a.pair_span) * 4;
  if (bsmem > 200 * 1024) return cudaErrorInvalidValue;
  auto kern = g == 4 ? k_pair_build<4> : k_pair_build<2>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((a.pair_npos + ch - 1) / ch), (unsigned)a.pair_npair, (unsigned)(a.beams ? a.nbeam : 1));
  kern<<<grid, 256, bsmem, s>>>(a);
  count_launches(1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const bool multi = a.beams && a.nbeam > 1;
  switch (a.cc * 2 + (multi ? 1 : 0)) {
    case 8: return launch_sum<4, false>(a, s);
    case 9: return launch_sum<4, true>(a, s);
    case 16: return launch_sum<8, false>(a, s);
    case 17: return launch_sum<8, true>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace hg
