// Tensor-core X-step (tcgen05, sm_103a): per channel, the Hermitian product of
// the input spectra accumulated over time (Correlation_core::integration_step,
// sfxc/src/correlation_core.cc:241-273) as a real Gram matrix on the 5th-
// generation tensor cores.
//
// Each spectrum value x is stored as two FP16 numbers, hi = fp16(s*x) and
// lo = fp16(s*x - hi) (s a power of two), so hi + lo carries ~22 bits.
// Spectra layout (written by the windowed FFT, tc_index): per row, 32 stream
// slots x [hi.re, hi.im, lo.re, lo.im] FP16 per channel, stored as one
// 128-byte line per (group of four channels, slot quad), so a channel's
// slots are eight 32-byte pieces 128 B apart.  One TMA box per channel and
// K-tile gathers them, with the 32-byte swizzle, into the canonical MN-major
// layout: atoms of 8 rows x 32 B (16 components), the eight M atoms 256 B
// apart, 8-row groups 2 KB apart.  The M index of a component is
// 4 * stream + {hi.re, hi.im, lo.re, lo.im}.  The MMA computes
// D = A A^T (128 x 128, FP32 accumulation in TMEM); summing the four hi/lo
// combinations of a stream pair gives the compensated product, and the
// epilogue forms
//   Re V(a,b) = sum over re-re and im-im pairs,  Im V(a,b) = im-re minus re-im
// with lane shuffles over the 4 TMEM lanes (D rows) of one stream.
//
// Persistent CTA per SM, 10 warps, warp-specialised, over groups of 2
// channels: warp 0 streams K-tiles with TMA (cp.async.bulk.tensor, 128-byte
// swizzle, 2 boxes of 16 KB per 32 KB stage, 4 stages) without stopping at
// group boundaries; warp 1 issues 2 channels x 4 MMAs (K = 16) per stage into
// one of two TMEM buffers (2 x 256 columns) and commits each stage to its
// "empty" barrier and each finished group to the buffer's "full" barrier;
// warps 2-9 (one per channel and TMEM lane quarter) read the finished buffer,
// add the visibilities to the accumulator (8 loads in flight per lane) and
// release the buffer, while the next group accumulates in the other one.  Every wait is bounded: on timeout the
// CTA records an error and stops, waits (bounded) for its loads and MMAs in
// flight, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include "device.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"

namespace sfxc {
namespace {
using namespace tc;

constexpr int kChan = 2;        // channels per group (one TMEM buffer)
constexpr int kRowsK = 64;      // FFT rows per K-tile
constexpr int kStages = 4;   // 129 KB of shared memory; 3 stages measured 17 % slower, 6 stages 3 %
constexpr int kThreads = 320;   // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int kChanTile = kRowsK * 256;       // one channel's K-tile: 64 rows x 128 components x 2 B
constexpr int kStageBytes = kChan * kChanTile;  // 32 KB per stage
constexpr uint32_t kBufCols = kChan * 128;      // TMEM columns per buffer
// One channel's K-tile: TMA box {16 components, 8 rows, 8 slot quads, 8 row
// groups, 1 channel group} = 16 KB at row group rg and channel group cg.
__device__ __forceinline__ void tma_load_tile(void *dst, const CUtensorMap *map, int rg, int cg, uint64_t *bar) {
  tma_load_5d(dst, map, 0, 0, 0, rg, cg, bar);
}

// Tensor maps of the four channels of a channel group (base offsets 32 B apart).
struct TcMaps {
  CUtensorMap m[4];
};

__global__ void __launch_bounds__(kThreads, 1)
    xcorr_tc_kernel(const __grid_constant__ TcMaps tmaps, int nrows, int K, int kpad, const int *__restrict__ blmap,
                    int npad, float inv_scale2, float2 *__restrict__ acc, int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);  // stages 1 KB aligned
  __shared__ uint64_t full[kStages], empty[kStages], tfull[2], tempty[2], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ngroups = (K + kChan - 1) / kChan;
  const int nkt = (nrows + kRowsK - 1) / kRowsK;
  // this CTA's groups: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int my_groups = blockIdx.x < ngroups ? (ngroups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  if (warp == 0) {
    tmem_alloc(&tmem_base, 512);
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 8);  // one arrival per epilogue warp
    }
    mbar_init(&done, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  volatile int *vfailed = &failed;

  if (tid == 0) {
    // ---- TMA producer: every K-tile of every group, one stage ring
    int last[kStages];
    for (int s = 0; s < kStages; s++) last[s] = -1;
    int it = 0;
    for (int i = 0; i < my_groups && !*vfailed; i++) {
      const int g = blockIdx.x + i * gridDim.x;
      for (int kt = 0; kt < nkt; kt++, it++) {
        const int s = it % kStages, n = it / kStages;
        if ((n > 0 && !mbar_wait(&empty[s], (n - 1) & 1)) || *vfailed) {
          *vfailed = 1;
          break;
        }
        mbar_expect_tx(&full[s], kStageBytes);
        uint8_t *st = base + s * kStageBytes;
#pragma unroll
        for (int c = 0; c < kChan; c++) {
          const int ch = g * kChan + c;
          tma_load_tile(st + c * kChanTile, &tmaps.m[ch & 3], kt * (kRowsK / 8), ch >> 2, &full[s]);
        }
        last[s] = it;
      }
    }
    // loads still in flight land before the CTA may exit
    for (int s = 0; s < kStages; s++)
      if (last[s] >= 0 && !mbar_wait(&full[s], (last[s] / kStages) & 1)) *vfailed = 1;
  } else if (tid == 32) {
    // ---- MMA issuer
    const uint32_t idesc = idesc_f16(128, 128);
    int it = 0;
    for (int i = 0; i < my_groups && !*vfailed; i++) {
      const int b = i & 1, u = i >> 1;
      if (u > 0 && !mbar_wait(&tempty[b], (u - 1) & 1)) {  // the epilogue has read buffer b
        *vfailed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      bool ok = true;
      for (int kt = 0; kt < nkt; kt++, it++) {
        const int s = it % kStages, n = it / kStages;
        if (!mbar_wait(&full[s], n & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem_u32(base + s * kStageBytes);
#pragma unroll
        for (int c = 0; c < kChan; c++) {
#pragma unroll
          for (int ks = 0; ks < kRowsK / 16; ks++) {
            // 16 K-rows = two 8-row groups of 2 KB; M atoms 256 B apart
            const uint64_t d = smem_desc(st + c * kChanTile + ks * 4096, 256, 2048);
            mma_f16(tmem + b * kBufCols + c * 128, d, d, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
          }
        }
        mma_commit(&empty[s]);
      }
      if (!ok) {
        *vfailed = 1;
        break;
      }
      mma_commit(&tfull[b]);  // the group's sums are complete when its MMAs are
    }
    mma_commit(&done);  // arrives once every MMA issued above has completed
  } else if (warp >= 2) {
    // ---- epilogue: warp w reads channel (w - 2) / 4 of the group, TMEM lanes
    // 32 (w % 4) .. + 31 (D rows)
    const int q = warp & 3, c = (warp - 2) >> 2, m = q * 32 + lane, a = m >> 2, p = m & 3;
    for (int i = 0; i < my_groups; i++) {
      const int b = i & 1, u = i >> 1;
      if (!mbar_wait(&tfull[b], u & 1)) {
        *vfailed = 1;
        break;
      }
      if (*vfailed) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int k = (blockIdx.x + i * gridDim.x) * kChan + c;
#pragma unroll 1
      for (int j = 0; j < 4; j++) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + b * kBufCols + c * 128 + j * 32, v);
        float re8[8], im8[8];
#pragma unroll
        for (int bb = 0; bb < 8; bb++) {
          const float A = v[4 * bb] + v[4 * bb + 2], B = v[4 * bb + 1] + v[4 * bb + 3];
          // row component p: 0 hi.re, 1 hi.im, 2 lo.re, 3 lo.im; columns likewise
          float re = (p & 1) ? B : A, im = (p & 1) ? A : -B;
          re += __shfl_xor_sync(0xffffffffu, re, 1);
          im += __shfl_xor_sync(0xffffffffu, im, 1);
          re += __shfl_xor_sync(0xffffffffu, re, 2);
          im += __shfl_xor_sync(0xffffffffu, im, 2);
          re8[bb] = re;
          im8[bb] = im;
        }
        if (p == 0 && k < K && a < npad) {
          // the 8 baselines' accumulator loads in flight together
          int mv[8];
          float2 o[8];
#pragma unroll
          for (int bb = 0; bb < 8; bb++) mv[bb] = j * 8 + bb < npad ? __ldg(blmap + a * npad + j * 8 + bb) : -1;
#pragma unroll
          for (int bb = 0; bb < 8; bb++)
            if (mv[bb] >= 0) o[bb] = acc[(int64_t)(mv[bb] >> 1) * kpad + k];
#pragma unroll
          for (int bb = 0; bb < 8; bb++)
            if (mv[bb] >= 0) {
              o[bb].x += re8[bb] * inv_scale2;
              o[bb].y += ((mv[bb] & 1) ? -im8[bb] : im8[bb]) * inv_scale2;
              acc[(int64_t)(mv[bb] >> 1) * kpad + k] = o[bb];
            }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);  // buffer b may be overwritten
    }
  }
  __syncthreads();
  if (!mbar_wait(&done, 0)) *vfailed = 1;  // no MMA in flight past this point
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (*vfailed && tid == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// Row-gathered tensor-core X-step: the same compensated Gram products, with
// each channel's FFT rows taken in the order of a per-channel row list, cut
// into segments that go to separate accumulators:
//   * pulsar binning (Correlation_core_pulsar::integration_step,
//     sfxc/src/correlation_core_pulsar.cc:101-146 with the bins of 210-238):
//     each channel's rows sorted by bin (pulsar_sort_kernel), one segment per
//     bin, the segment's Gram added to acc[bin];
//   * jobs of 33 to 64 streams (S = 64 slots): rows in order, one segment.
// Warps 0-3 gather K-tiles of up to 64 listed rows with 16-byte cp.async
// straight into the 32-byte-swizzled MN-major layout that the TMA kernel's
// boxes produce (list entries of -1 read as zero rows) and publish each tile
// after a proxy fence; warp 4 issues the MMAs -- per 16 rows, block I = 0
// (and 1 for S = 64): M = 128 rows of components from 128 I, N = the
// components from 128 I to the last stream (FP32 accumulation in the
// segment's TMEM buffer); warps 5-12 add each finished buffer to its
// accumulator while the next segments accumulate in the other buffers.
// Every wait is bounded: on timeout the CTA records an error and stops,
// waits (bounded) for its copies and MMAs in flight, frees its TMEM and
// returns.
template <int S>
struct GatherShape {
  static constexpr int kRows = 64;                       // rows per K-tile
  static constexpr int kGroupBytes = (S / 4) * 256;      // one 8-row K group: S/4 atoms of 8 rows x 32 B
  static constexpr int kStageBytes = 8 * kGroupBytes;    // 16 KB (S = 32) or 32 KB (S = 64)
  static constexpr int kStages = 131072 / kStageBytes;   // 128 KB of stages: one CTA per SM
  static constexpr int kProducers = 128;                 // warps 0-3
  static constexpr int kThreads = 416;                   // + warp 4 (MMA) + warps 5-12 (epilogue)
  static constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024;
};

struct GatherArgs {
  const uint8_t *spec;  // TC layout with S slots
  int nrows;            // rows in the buffer; list entries outside [0, nrows) read as zeros
  int kpad, K, nstreams, npad, nbl, nbins;
  const int *rowlist;   // per channel list_len entries (row or -1); NULL: the rows in order
  int list_len;
  const int2 *segs;     // per (channel, bin): first list entry, entries (a multiple of 16); NULL: one segment
  const int *blmap;
  float inv_scale2;
  float2 *acc;          // [bin][baseline][kpad]
  int *err;
  int n0, n1, col1;     // MMA N of blocks 0 and 1 (n1 = 0: one block), TMEM column of block 1
  int buf_stride, nbuf; // TMEM columns per buffer, number of buffers
  int accumulate;       // 0: every (bin, channel) segment is the only one of its launch and is stored as it is
};

constexpr int kMaxBufs = 8;

__device__ __forceinline__ int2 gather_seg(const GatherArgs &g, int ch, int bin) {
  if (!g.segs) return make_int2(0, (g.nrows + 15) & ~15);
  return g.segs[(size_t)ch * g.nbins + bin];
}

// One K-tile of a segment.
struct GTile {
  int ch, bin, e0, rows;  // channel, bin, first list entry, rows (a multiple of 16)
  bool first, last;       // first / last tile of its segment
};

// The K-tiles of this CTA in processing order: channel groups of four
// (group blockIdx.x, then + gridDim.x); within a group bin by bin; within a
// bin the group's four channels; within a segment 64 rows at a time.  The
// four channels of a group read the four 32-byte pieces of the same 128-byte
// spectra lines and write the same 32-byte accumulator sectors close together
// in time.  Every role of the kernel walks the same sequence.
struct GWalk {
  int grp, bin, c, t0;
  int2 sg;
  __device__ void init() {
    grp = blockIdx.x;
    bin = 0;
    c = -1;
    t0 = 0;
    sg = make_int2(0, 0);
  }
  __device__ bool next(const GatherArgs &g, int ngroups, GTile &t) {
    if (t0 + 64 < sg.y) {  // more rows in the current segment
      t0 += 64;
    } else {
      for (;;) {  // the next non-empty segment
        if (++c == 4) {
          c = 0;
          if (++bin == g.nbins) {
            bin = 0;
            grp += gridDim.x;
          }
        }
        if (grp >= ngroups) return false;
        const int ch = 4 * grp + c;
        if (ch >= g.K) continue;
        sg = gather_seg(g, ch, bin);
        if (sg.y > 0) break;
      }
      t0 = 0;
    }
    t.ch = 4 * grp + c;
    t.bin = bin;
    t.e0 = sg.x + t0;
    t.rows = min(64, sg.y - t0);
    t.first = t0 == 0;
    t.last = t0 + 64 >= sg.y;
    return true;
  }
};

template <int S>
__global__ void __launch_bounds__(GatherShape<S>::kThreads, 1) xcorr_tc_gather_kernel(const __grid_constant__ GatherArgs g) {
  using G = GatherShape<S>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);  // stages 1 KB aligned
  __shared__ uint64_t full[G::kStages], empty[G::kStages], tfull[kMaxBufs], tempty[kMaxBufs], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 4) tmem_alloc(&tmem_base, 512);
  if (tid == 0) {
    for (int s = 0; s < G::kStages; s++) {
      mbar_init(&full[s], G::kProducers);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < kMaxBufs; b++) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 8);  // one arrival per epilogue warp
    }
    mbar_init(&done, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base;
  volatile int *vfailed = &failed;
  const int ngroups = (g.K + 3) / 4;
  GWalk walk;
  walk.init();
  GTile t;

  if (tid < G::kProducers) {
    // ---- producers: thread tid copies, for every row j = j0 + RP i of a
    // tile, the 16-byte half h of slot quad q (quads one 128-byte line
    // apart); the row-list entries of the next tile load while the current
    // tile is issued
    constexpr int CPR = S / 2;               // 16-byte chunks per row
    constexpr int RP = G::kProducers / CPR;  // rows per pass
    constexpr int E = G::kRows / RP;         // rows per thread and tile
    const int j0 = tid / CPR, q = (tid % CPR) >> 1, h = tid & 1;
    const uint32_t soff = q * 256;
    const int64_t rstride = (int64_t)g.kpad * S * 8;  // bytes per row
    int rcur[E], rnxt[E];
    auto load_rows = [&](const GTile &x, int(&r)[E]) {
      const int *list = g.rowlist ? g.rowlist + (size_t)x.ch * g.list_len : nullptr;
#pragma unroll
      for (int i = 0; i < E; i++) {
        const int j = j0 + RP * i;
        r[i] = j < x.rows ? (list ? __ldg(list + x.e0 + j) : x.e0 + j) : -2;
      }
    };
    GTile cur, nxt;
    bool have = walk.next(g, ngroups, cur);
    if (have) load_rows(cur, rcur);
    int it = 0;
    while (have) {
      const bool have_next = walk.next(g, ngroups, nxt);
      if (have_next) load_rows(nxt, rnxt);
      const int s = it % G::kStages, n = it / G::kStages;
      if ((n > 0 && !mbar_wait(&empty[s], (n - 1) & 1)) || *vfailed) {
        *vfailed = 1;
        break;
      }
      const uint32_t st = smem_u32(base + s * G::kStageBytes);
      const uint8_t *chbase = g.spec + (tc_index(0, g.kpad, cur.ch, 4 * q, S) * 8 + 16 * h);
#pragma unroll
      for (int i = 0; i < E; i++) {
        if (rcur[i] == -2) break;  // past the tile's rows (the rows grow with i)
        const int j = j0 + RP * i, row = rcur[i];
        const bool ok = row >= 0 && row < g.nrows;
        cp_async16(st + (j >> 3) * G::kGroupBytes + soff + sw32_offset(j & 7, h), ok ? chbase + row * rstride : g.spec,
                   ok ? 16u : 0u);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
      if (it > 0) {  // the previous tile has landed: publish it to the tensor cores
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&full[(it - 1) % G::kStages]);
      }
      it++;
      cur = nxt;
#pragma unroll
      for (int i = 0; i < E; i++) rcur[i] = rnxt[i];
      have = have_next;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (it > 0) mbar_arrive(&full[(it - 1) % G::kStages]);
  } else if (tid == 4 * 32) {
    // ---- MMA issuer
    const uint32_t id0 = idesc_f16(128, g.n0), id1 = idesc_f16(128, g.n1 > 0 ? g.n1 : 16);
    int it = 0, sgn = 0;
    uint32_t d0 = tmem;
    while (walk.next(g, ngroups, t)) {
      const int b = sgn % g.nbuf, u = sgn / g.nbuf;
      if (t.first) {
        if ((u > 0 && !mbar_wait(&tempty[b], (u - 1) & 1)) || *vfailed) {  // the epilogue has read buffer b
          *vfailed = 1;
          break;
        }
        fence_after_sync();
        d0 = tmem + (uint32_t)(b * g.buf_stride);
      }
      const int s = it % G::kStages, n = it / G::kStages;
      if (!mbar_wait(&full[s], n & 1)) {
        *vfailed = 1;
        break;
      }
      fence_after_sync();
      const uint32_t st = smem_u32(base + s * G::kStageBytes);
      for (int ks = 0; ks < t.rows / 16; ks++) {
        const uint32_t acc_flag = (!t.first || ks > 0) ? 1u : 0u;
        // 16 K rows = two 8-row groups; MN atoms 256 B apart; block 1 starts 8 atoms in
        const uint64_t a0 = smem_desc(st + ks * 2 * G::kGroupBytes, 256, G::kGroupBytes);
        mma_f16(d0, a0, a0, id0, acc_flag);
        if (g.n1 > 0) {
          const uint64_t a1 = smem_desc(st + ks * 2 * G::kGroupBytes + 2048, 256, G::kGroupBytes);
          mma_f16(d0 + (uint32_t)g.col1, a1, a1, id1, acc_flag);
        }
      }
      mma_commit(&empty[s]);
      it++;
      if (t.last) {
        mma_commit(&tfull[b]);  // the segment's sums are complete when its MMAs are
        sgn++;
      }
    }
    mma_commit(&done);  // arrives once every MMA issued above has completed
  } else if (warp >= 5) {
    // ---- epilogue: warp w reads TMEM lane quarter q = w % 4 (D rows 32 q ..
    // 32 q + 31 of each block) and every other 16-column chunk
    const int q = warp & 3, half = (warp - 5) >> 2;
    const int m = q * 32 + lane, p = m & 3;
    int sgn = 0;
    while (walk.next(g, ngroups, t)) {
      if (!t.last) continue;
      const int b = sgn % g.nbuf, u = sgn / g.nbuf;
      if (!mbar_wait(&tfull[b], u & 1) || *vfailed) {
        *vfailed = 1;
        break;
      }
      fence_after_sync();
      float2 *accb = g.acc + (size_t)t.bin * g.nbl * g.kpad + t.ch;
      for (int I = 0; I < (g.n1 > 0 ? 2 : 1); I++) {
        if (32 * I + 8 * q >= g.nstreams) continue;  // no stream in this lane quarter
        const int a = 32 * I + (m >> 2);
        const int nI = I ? g.n1 : g.n0;
        const uint32_t col = (uint32_t)(b * g.buf_stride + (I ? g.col1 : 0));
#pragma unroll 1
        for (int chunk = half; chunk < nI / 16; chunk += 2) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + col + 16 * chunk, v);
          float re4[4], im4[4];
#pragma unroll
          for (int bb = 0; bb < 4; bb++) {
            const float A = v[4 * bb] + v[4 * bb + 2], B = v[4 * bb + 1] + v[4 * bb + 3];
            // row component p: 0 hi.re, 1 hi.im, 2 lo.re, 3 lo.im; columns likewise
            float re = (p & 1) ? B : A, im = (p & 1) ? A : -B;
            re += __shfl_xor_sync(0xffffffffu, re, 1);
            im += __shfl_xor_sync(0xffffffffu, im, 1);
            re += __shfl_xor_sync(0xffffffffu, re, 2);
            im += __shfl_xor_sync(0xffffffffu, im, 2);
            re4[bb] = re;
            im4[bb] = im;
          }
          if (p == 0 && a < g.nstreams) {
            int mv[4];
#pragma unroll
            for (int bb = 0; bb < 4; bb++) {
              const int bs = 32 * I + 4 * chunk + bb;
              mv[bb] = bs < g.nstreams ? __ldg(g.blmap + a * g.npad + bs) : -1;
            }
            float2 o[4];
            if (g.accumulate) {
#pragma unroll
              for (int bb = 0; bb < 4; bb++)
                if (mv[bb] >= 0) o[bb] = accb[(size_t)(mv[bb] >> 1) * g.kpad];
            } else {
#pragma unroll
              for (int bb = 0; bb < 4; bb++) o[bb] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int bb = 0; bb < 4; bb++)
              if (mv[bb] >= 0) {
                o[bb].x += re4[bb] * g.inv_scale2;
                o[bb].y += ((mv[bb] & 1) ? -im4[bb] : im4[bb]) * g.inv_scale2;
                accb[(size_t)(mv[bb] >> 1) * g.kpad] = o[bb];
              }
          }
        }
      }
      fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);  // buffer b may be overwritten
      sgn++;
    }
  }
  __syncthreads();
  if (!mbar_wait(&done, 0)) *vfailed = 1;  // no MMA in flight past this point
  fence_after_sync();
  __syncthreads();
  if (*vfailed && tid == 0) atomicExch(g.err, 1);
  fence_before_sync();
  __syncthreads();
  if (warp == 4) {
    fence_after_sync();
    tmem_dealloc(tmem, 512);
  }
}

// Rows of each channel sorted stably by pulsar bin, each bin's run padded
// with -1 entries to a multiple of 16 rows: rowlist[ch][list_len] and
// segs[ch][bin] = (first entry, entries).  bins: [channel][row].  One warp
// per channel; shared counters per warp.
__global__ void __launch_bounds__(128) pulsar_sort_kernel(const int16_t *__restrict__ bins, int nrows, int K,
                                                          int nbins, int list_len, int *__restrict__ rowlist,
                                                          int2 *__restrict__ segs) {
  extern __shared__ int cnt[];  // per warp: count[nbins], cursor[nbins]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ch = blockIdx.x * 4 + w;
  if (ch >= K) return;  // whole warps
  int *count = cnt + w * 2 * nbins, *cursor = count + nbins;
  for (int b = lane; b < nbins; b += 32) count[b] = 0;
  __syncwarp();
  const int16_t *br = bins + (size_t)ch * nrows;
  for (int r = lane; r < nrows; r += 32) atomicAdd(&count[br[r]], 1);
  __syncwarp();
  if (lane == 0) {
    int pos = 0;
    for (int b = 0; b < nbins; b++) {
      const int len = (count[b] + 15) & ~15;
      segs[(size_t)ch * nbins + b] = make_int2(pos, len);
      cursor[b] = pos;
      pos += len;
    }
  }
  __syncwarp();
  int *list = rowlist + (size_t)ch * list_len;
  for (int b = lane; b < nbins; b += 32)  // padding entries of each run
    for (int e = cursor[b] + count[b]; e < cursor[b] + ((count[b] + 15) & ~15); e++) list[e] = -1;
  __syncwarp();
  for (int r0 = 0; r0 < nrows; r0 += 32) {
    const int r = r0 + lane;
    const int b = r < nrows ? br[r] : -1;
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(same & ((1u << lane) - 1u));
    const int pos = b >= 0 ? cursor[b] + rank : 0;
    __syncwarp();
    if (b >= 0) {
      list[pos] = r;
      if (rank == 0) cursor[b] = pos + __popc(same);
    }
    __syncwarp();
  }
}

}  // namespace

size_t xcorr_tc_smem_bytes() { return kStages * (size_t)kStageBytes + 1024; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

cudaError_t launch_xcorr_tc(const void *spec, int nrows, int kpad, int K, const int *blmap, int npad,
                            float inv_scale2, float2 *acc, int *err, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  // per channel of a group (base + 32 B each): 16 components of a slot quad,
  // rows within an 8-row group (kpad * 256 B apart), the 8 slot quads (128 B
  // apart), 8-row groups, channel groups (1 KB apart).  Rows from nrows up to
  // the next multiple of 8 must be zero in the buffer (the caller clears
  // them); row groups past the end read as zeros.
  if (kpad % 4 != 0) return cudaErrorInvalidValue;
  TcMaps maps;
  const cuuint64_t R = (cuuint64_t)kpad * 256;
  const cuuint64_t dims[5] = {16, 8, 8, (cuuint64_t)(nrows + 7) / 8, (cuuint64_t)kpad / 4};
  const cuuint64_t strides[4] = {R, 128, 8 * R, 1024};
  const cuuint32_t box[5] = {16, 8, 8, (cuuint32_t)kRowsK / 8, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  for (int cc = 0; cc < 4; cc++)
    if (enc(&maps.m[cc], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, static_cast<char *>(const_cast<void *>(spec)) + 32 * cc,
            dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  const size_t smem = xcorr_tc_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(xcorr_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
  const int ngroups = (K + kChan - 1) / kChan;
  xcorr_tc_kernel<<<std::min(ngroups, nsm), kThreads, smem, st>>>(maps, nrows, K, kpad, blmap, npad, inv_scale2, acc,
                                                                   err);
  return cudaGetLastError();
}

template <int S>
static cudaError_t launch_gather(const GatherArgs &g, cudaStream_t st) {
  using G = GatherShape<S>;
  cudaError_t e = cudaFuncSetAttribute(xcorr_tc_gather_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)G::kSmem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
  xcorr_tc_gather_kernel<S><<<std::min((g.K + 3) / 4, nsm), G::kThreads, G::kSmem, st>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_xcorr_tc_gather(const void *spec, int slots, int nrows, int kpad, int K, int nstreams,
                                   const int *blmap, int npad, int nbl, int nbins, const int *rowlist, int list_len,
                                   const int2 *segs, float inv_scale2, float2 *acc, int *err, cudaStream_t st) {
  if (nrows <= 0 || K <= 0) return cudaSuccess;
  if ((slots != kTcSlots && slots != kTcSlotsWide) || nstreams > slots || nstreams <= 0)
    return cudaErrorInvalidValue;
  GatherArgs g;
  g.spec = static_cast<const uint8_t *>(spec);
  g.nrows = nrows;
  g.kpad = kpad;
  g.K = K;
  g.nstreams = nstreams;
  g.npad = npad;
  g.nbl = nbl;
  g.nbins = rowlist ? nbins : 1;
  g.rowlist = rowlist;
  g.list_len = list_len;
  g.segs = rowlist ? segs : nullptr;
  g.blmap = blmap;
  g.inv_scale2 = inv_scale2;
  g.acc = acc;
  g.err = err;
  auto up16 = [](int x) { return (x + 15) & ~15; };
  auto up32 = [](int x) { return (x + 31) & ~31; };
  const int comps = 4 * nstreams;
  g.n0 = up16(std::min(comps, 256));
  g.n1 = comps > 128 ? up16(comps - 128) : 0;
  g.col1 = up32(g.n0);
  g.buf_stride = g.col1 + up32(g.n1);
  g.nbuf = std::min(kMaxBufs, 512 / g.buf_stride);
  // with a row list (pulsar binning: the whole integration in one launch) each
  // (bin, channel) segment is the only one of its accumulator entries
  g.accumulate = rowlist ? 0 : 1;
  if (slots == kTcSlots) return launch_gather<kTcSlots>(g, st);
  return launch_gather<kTcSlotsWide>(g, st);
}

void launch_pulsar_sort(const int16_t *bins, int nrows, int K, int nbins, int list_len, int *rowlist, int2 *segs,
                        cudaStream_t st) {
  const size_t smem = (size_t)4 * 2 * nbins * sizeof(int);
  if (smem > 48 * 1024) cudaFuncSetAttribute(pulsar_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  pulsar_sort_kernel<<<(K + 3) / 4, 128, smem, st>>>(bins, nrows, K, nbins, list_len, rowlist, segs);
}

}  // namespace sfxc
