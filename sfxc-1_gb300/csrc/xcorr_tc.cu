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

namespace sfxc {
namespace {

constexpr int kChan = 2;        // channels per group (one TMEM buffer)
constexpr int kRowsK = 64;      // FFT rows per K-tile
constexpr int kStages = 4;   // 129 KB of shared memory; 3 stages measured 17 % slower, 6 stages 3 %
constexpr int kThreads = 320;   // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int kChanTile = kRowsK * 256;       // one channel's K-tile: 64 rows x 128 components x 2 B
constexpr int kStageBytes = kChan * kChanTile;  // 32 KB per stage
constexpr uint32_t kBufCols = kChan * 128;      // TMEM columns per buffer
constexpr unsigned long long kSpinLimit = 200000000ull;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// SM100 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading
// byte offset >> 4 (16-29), stride byte offset >> 4 (32-45), version 1
// (bit 46), base offset 0, layout type SWIZZLE_32B = 6 (bits 61-63).  For the
// MN-major operand the leading offset steps between M atoms, the stride
// offset between 8-row K groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)6 << 61;
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One channel's K-tile: TMA box {16 components, 8 rows, 8 slot quads, 8 row
// groups, 1 channel group} = 16 KB at row group rg and channel group cg.
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, int rg, int cg, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(0), "r"(rg), "r"(cg), "r"(smem_u32(bar))
      : "memory");
}

// Tensor maps of the four channels of a channel group (base offsets 32 B apart).
struct TcMaps {
  CUtensorMap m[4];
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

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
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
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
          tma_load_5d(st + c * kChanTile, &tmaps.m[ch & 3], kt * (kRowsK / 8), ch >> 2, &full[s]);
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
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

}  // namespace sfxc
