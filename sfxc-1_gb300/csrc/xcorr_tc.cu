// Tensor-core X-step (tcgen05, sm_103a): per channel, the Hermitian product of
// the input spectra accumulated over time (Correlation_core::integration_step,
// sfxc/src/correlation_core.cc:241-273) as a real Gram matrix on the 5th-
// generation tensor cores.
//
// Each spectrum value x is stored as two FP16 numbers, hi = fp16(s*x) and
// lo = fp16(s*x - hi) (s a power of two), so hi + lo carries ~22 bits.  For
// one channel, the 128 "rows" of A are the components [hi.re, hi.im] of 32
// inputs followed by [lo.re, lo.im]; A has one column per FFT (time).  The MMA
// computes D = A A^T (128x128, FP32 accumulation in TMEM); summing its four
// 64x64 quadrants gives (hi+lo)(hi+lo)^T exactly as products of the FP16
// parts, i.e. the compensated product, and the epilogue forms
//   Re V(a,b) = G[2a][2b] + G[2a+1][2b+1],  Im V(a,b) = G[2a+1][2b] - G[2a][2b+1].
//
// CTA: 4 channels (4 x 128 TMEM columns), 256 threads.  K-tiles of 64 FFTs,
// double buffered in shared memory in the canonical MN-major 128-byte-swizzle
// layout (per channel: two 64-component atoms of 64 rows x 128 B).  All
// threads stage a tile (global loads, swizzled stores, async-proxy fence);
// thread 0 issues 4 channels x 4 MMAs (K = 16 each) and commits them to the
// stage's mbarrier.  Waits are bounded: on timeout the CTA records an error,
// skips its output, frees its TMEM and returns.
#include <cstdint>
#include <cuda_fp16.h>

#include "device.cuh"
#include "kernels.hpp"

namespace sfxc {
namespace {

constexpr int kChan = 4;        // channels per CTA
constexpr int kRowsK = 64;      // FFT rows per K-tile
constexpr int kThreads = 256;
constexpr int kAtomBytes = kRowsK * 128;      // one 64-component atom of a K-tile
constexpr int kChanTile = 2 * kAtomBytes;     // hi + lo atoms of one channel
constexpr int kStageBytes = kChan * kChanTile;  // 64 KB per stage
constexpr unsigned long long kSpinLimit = 200000000ull;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// SM100 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading
// byte offset >> 4 (16-29), stride byte offset >> 4 (32-45), version 1
// (bit 46), base offset 0, layout type SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B FP16
// (formats 0), A and B MN-major (bits 15, 16), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | (1u << 15) | (1u << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the phase with the given parity: gives up after kWaitNs of
// wall time (and after kSpinLimit polls), returning false.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const uint64_t t0 = globaltimer_ns();
  for (unsigned long long i = 0; i < kSpinLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255) == 255 && globaltimer_ns() - t0 > kWaitNs) return false;
  }
  return false;
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive FP32 columns of the warp's TMEM subpartition.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Byte offset of component m (0..127) at K-row k in one channel's tile.
__device__ __forceinline__ uint32_t tile_offset(int m, int k) {
  const int atom = m >> 6, mm = m & 63;
  return (uint32_t)(atom * kAtomBytes + (k >> 3) * 1024 + (k & 7) * 128 + ((((mm >> 3) ^ (k & 7))) << 4) +
                    (mm & 7) * 2);
}

__global__ void __launch_bounds__(kThreads, 1)
    xcorr_tc_kernel(const uint2 *__restrict__ spec, int nrows_total, int kpad, int nstreams, int nrows, int K,
                    const int *__restrict__ blmap, int npad, float inv_scale2, float2 *__restrict__ acc,
                    int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-B aligned dynamic shared memory: two stages, then epilogue staging
  uint8_t *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  uint8_t *stage[2] = {base, base + kStageBytes};
  float *stg = reinterpret_cast<float *>(base);  // reused after the MMAs: [128][65]
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int k0 = blockIdx.x * kChan;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = idesc_f16(128, 128);
  const int nkt = (nrows + kRowsK - 1) / kRowsK;

  for (int kt = 0; kt < nkt; kt++) {
    const int s = kt & 1;
    if (kt >= 2) {
      if (!mbar_wait(&mbar[s], ((kt - 2) >> 1) & 1)) failed = 1;
    }
    __syncthreads();
    if (failed) break;
    // ---- stage the K-tile: (stream, row) pairs, 4 channels x (hi, lo) each
    uint8_t *st = stage[s];
    for (int e = tid; e < 32 * kRowsK; e += kThreads) {
      const int sidx = e & 31, r = e >> 5;
      const int row = kt * kRowsK + r;
      uint2 v[kChan];
#pragma unroll
      for (int c = 0; c < kChan; c++) v[c] = make_uint2(0u, 0u);
      if (sidx < nstreams && row < nrows) {
        const uint2 *src = spec + ((int64_t)sidx * nrows_total + row) * kpad + k0;
#pragma unroll
        for (int c = 0; c < kChan; c++)
          if (k0 + c < K) v[c] = src[c];
      }
#pragma unroll
      for (int c = 0; c < kChan; c++) {
        uint8_t *t = st + c * kChanTile;
        *reinterpret_cast<uint32_t *>(t + tile_offset(2 * sidx, r)) = v[c].x;       // hi re, hi im
        *reinterpret_cast<uint32_t *>(t + tile_offset(64 + 2 * sidx, r)) = v[c].y;  // lo re, lo im
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c = 0; c < kChan; c++) {
        const uint32_t a0 = smem_u32(st + c * kChanTile);
#pragma unroll
        for (int ks = 0; ks < kRowsK / 16; ks++) {
          // 16 K-rows = two 8-row groups of 1024 B; atoms (hi, lo) kAtomBytes apart
          const uint64_t d = smem_desc(a0 + ks * 2048, kAtomBytes, 1024);
          mma_f16(tmem + c * 128, d, d, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
        }
      }
      mma_commit(&mbar[s]);
    }
  }
  // ---- wait for the last tile's MMAs (the commit covers all earlier ones)
  if (!failed && nkt > 0) {
    if (!mbar_wait(&mbar[(nkt - 1) & 1], ((nkt - 1) >> 1) & 1)) failed = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    // ---- epilogue per channel: quadrant sums via shared memory, then baselines
    for (int c = 0; c < kChan; c++) {
      const int k = k0 + c;
      if (warp < 4) {
        const int m = warp * 32 + lane;  // TMEM lane = D row
        float lo[32], hi[32];
        for (int q0 = 0; q0 < 64; q0 += 32) {
          const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + c * 128;
          tmem_ld32(ta + q0, lo);
          tmem_ld32(ta + 64 + q0, hi);
#pragma unroll
          for (int q = 0; q < 32; q++) stg[m * 65 + q0 + q] = lo[q] + hi[q];
        }
      }
      __syncthreads();
      if (k < K) {
        for (int p = tid; p < npad * npad; p += kThreads) {
          const int i = p / npad, j = p % npad;
          const int mapv = blmap[i * npad + j];
          if (mapv < 0 || i >= 32 || j >= 32) continue;
          auto G = [&](int a, int b) { return stg[a * 65 + b] + stg[(a + 64) * 65 + b]; };
          const float re = (G(2 * i, 2 * j) + G(2 * i + 1, 2 * j + 1)) * inv_scale2;
          float im = (G(2 * i + 1, 2 * j) - G(2 * i, 2 * j + 1)) * inv_scale2;
          if (mapv & 1) im = -im;
          float2 *dst = acc + (int64_t)(mapv >> 1) * kpad + k;
          float2 o = *dst;
          o.x += re;
          o.y += im;
          *dst = o;
        }
      }
      __syncthreads();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

}  // namespace

size_t xcorr_tc_smem_bytes() { return 2 * (size_t)kStageBytes + 1024; }

void launch_xcorr_tc(const void *spec, int nrows_total, int kpad, int nstreams, int nrows, int K, const int *blmap,
                     int npad, float inv_scale2, float2 *acc, int *err, cudaStream_t st) {
  const size_t smem = xcorr_tc_smem_bytes();
  cudaFuncSetAttribute(xcorr_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  xcorr_tc_kernel<<<(K + kChan - 1) / kChan, kThreads, smem, st>>>(reinterpret_cast<const uint2 *>(spec),
                                                                  nrows_total, kpad, nstreams, nrows, K, blmap, npad,
                                                                  inv_scale2, acc, err);
}

}  // namespace sfxc
