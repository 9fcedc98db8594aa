// Compute peaks of the GPU the library runs on, the denominators of the
// compute rooflines: FP32 fused multiply-adds on the CUDA cores, and FP16
// tensor-core MMAs with FP32 accumulation (tcgen05.mma kind::f16, M = 128,
// N = 256, K = 16, operands in shared memory).  Each is one short kernel timed
// with CUDA events; nothing here changes a clock or any other device setting.
#include <algorithm>
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "sfxc_gpu.h"
#include "tc_ptx.cuh"

namespace sfxc {
namespace {
using namespace tc;

constexpr int kFmaChains = 16;

// 16 independent FMA chains per thread; the sum is stored only on an
// impossible value, which keeps every chain live.
__global__ void __launch_bounds__(256) fp32_peak_kernel(float *out, int iters, float b, float c) {
  float a[kFmaChains];
#pragma unroll
  for (int i = 0; i < kFmaChains; i++) a[i] = threadIdx.x * 1e-3f + i;
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < kFmaChains; i++) a[i] = fmaf(a[i], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kFmaChains; i++) s += a[i];
  if (s == -1.2345f) out[threadIdx.x] = s;
}

constexpr int kTcSmem = 120 * 1024;  // more than half an SM's shared memory: one CTA per SM

// One CTA per SM: thread 0 issues `iters` MMAs of 128 x 256 x 16 into two
// alternating TMEM accumulators and waits (bounded) for their completion.
__global__ void __launch_bounds__(128, 1) tc_peak_kernel(int iters, int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x;
  // A: 128 x 16 FP16 (4 KB), B: 256 x 16 (8 KB), 32-byte-swizzled MN-major; small values
  __half *h = reinterpret_cast<__half *>(base);
  for (int i = tid; i < 6144; i += blockDim.x) h[i] = __float2half(0.001f * (float)((i * 37) % 17 - 8));
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if ((tid >> 5) == 0) tmem_alloc(&tmem_base, 512);
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base;
  if (tid == 0) {
    const uint32_t a = smem_u32(base), b = a + 4096;
    const uint64_t ad = smem_desc(a, 256, 2048), bd = smem_desc(b, 256, 4096);
    const uint32_t id = idesc_f16(128, 256);
#pragma unroll 1
    for (int it = 0; it < iters; it++) mma_f16(tmem + (uint32_t)((it & 1) * 256), ad, bd, id, it >= 2 ? 1u : 0u);
    mma_commit(&bar);
    if (!mbar_wait(&bar, 0)) atomicExch(err, 1);
  }
  __syncthreads();
  fence_after_sync();
  if ((tid >> 5) == 0) tmem_dealloc(tmem, 512);
}

}  // namespace
}  // namespace sfxc

extern "C" int sfxc_gpu_measure_peaks(int32_t device, double *out4) {
  using namespace sfxc;
  if (!out4) return SFXC_GPU_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return SFXC_GPU_ECUDA;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || nsm <= 0)
    return SFXC_GPU_ECUDA;
  float *dout = nullptr;
  int *derr = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&dout, 1024 * sizeof(float)) != cudaSuccess) return SFXC_GPU_ECUDA;
  if (cudaMalloc(&derr, sizeof(int)) != cudaSuccess) {
    cudaFree(dout);
    return SFXC_GPU_ECUDA;
  }
  cudaMemset(derr, 0, sizeof(int));
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto best_ms = [&](auto launch) {
    launch();  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
      cudaEventRecord(e0);
      launch();
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, ms);
    }
    return best;
  };
  // FP32: 8 CTAs of 256 threads per SM, 16 chains x iters FMAs per thread
  const int fiters = 80000;
  const float fms = best_ms([&] { fp32_peak_kernel<<<8 * nsm, 256>>>(dout, fiters, 0.9999999f, 1e-7f); });
  const double fflop = 2.0 * kFmaChains * fiters * 256.0 * 8 * nsm;
  // tensor cores: one CTA per SM
  cudaFuncSetAttribute(tc_peak_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  const int titers = 160000;
  const float tms = best_ms([&] { tc_peak_kernel<<<nsm, 128, kTcSmem>>>(titers, derr); });
  const double tflop = 2.0 * 128 * 256 * 16 * (double)titers * nsm;
  int herr = 0;
  cudaError_t ce = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dout);
  cudaFree(derr);
  if (ce != cudaSuccess || cudaGetLastError() != cudaSuccess) return SFXC_GPU_ECUDA;
  if (herr) return SFXC_GPU_ECUDA;
  out4[0] = fflop / (fms * 1e-3) / 1e12;
  out4[1] = tflop / (tms * 1e-3) / 1e12;
  out4[2] = fms;
  out4[3] = tms;
  return SFXC_GPU_OK;
}
