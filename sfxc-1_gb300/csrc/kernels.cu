// CUDA kernels of the correlator-node path (sm_103a).
//
//   fstep_block_kernel   unpack (plan segments + 1/2-bit lookup) -> rfft(256)
//                        -> fractional-delay phase ramp -> complex ifft(256)
//                        -> fringe rotation; 16 threads per pair of blocks.
//                        Delay_correction::fractional_bit_shift / fringe_stopping
//                        (sfxc/src/delay_correction.cc:82-184) on the unpacked
//                        samples of Bit2float_worker (sfxc/src/bit2float_worker.cc:327-425).
//   window_fft_kernel    window, sideband flip, real FFT of 2M samples, channel
//                        selection (delay_correction.cc:57-75); M/16 threads per row.
// Both FFT stages are the register-resident radix-16 transforms of fft_reg.cuh.
//   bitstat_kernel       per-code sample counts with cal-diode on/off split, from
//                        popcounts (bit_statistics.cc:36-47, bit2float_worker.cc:341-346).
//   xcorr_f32_kernel     X-step on CUDA cores, 4x4 stream tiles per thread
//                        (Correlation_core::integration_step, correlation_core.cc:241-273).
//   pulsar_bins_kernel / xcorr_f32_pulsar  bin per (FFT, channel) in FP64 and binned
//                        accumulation (correlation_core_pulsar.cc:210-238).
//   norm_* kernels       Correlation_core::integration_normalize (275-314).
#include <algorithm>
#include <cstdio>

#include "device.cuh"
#include "fft_reg.cuh"
#include "kernels.hpp"

namespace sfxc {

// ------------------------------------------------------------------------
// F-step, stage 1: 16 threads per pair of 256-sample blocks.  One forward
// 256-point complex FFT of x_b + i x_{b+1} gives both real spectra
// (X[k] +/- conj X[256-k]); per block: DC and Nyquist halved, phase ramp
// exp(-i (c + k l)) on k <= 128, upper half zero, inverse 256-point FFT,
// fringe rotation of the real part.  tw holds exp(-2 pi i m / 256), m < 256.
//
// Samples n of the pair's two blocks written as xs[n] and xs[256 + n] by this
// half warp -> v[r] = (x_b[t + 16 r], x_b+1[t + 16 r]).  Only the half warp
// synchronises (the other may be on another path).
__device__ __forceinline__ void pair_from_scratch(float2 (&v)[16], const float *xs, int t) {
  const unsigned half = (threadIdx.x & 16) ? 0xFFFF0000u : 0x0000FFFFu;
  __syncwarp(half);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = make_float2(xs[t + 16 * r], xs[kNd + t + 16 * r]);
  __syncwarp(half);  // the FFT's first pass writes the scratch
}

// Pair (bl0, bl0 + 1) of a stream's blocks (indices from the stream's block0)
// by the 16 threads t = 0..15 of a half warp, with a scratch of kFsScratch
// float2; blocks at or past n_blocks give no output.  The
// result goes through store(block, sample, value).  Both half warps of a warp
// must call this together (warp barriers).
constexpr int kFsScratch = kNd + kNd / 16 + 9 * 16;
template <class Store>
__device__ __forceinline__ void fstep_pair(const StreamDev &s, int bl0, int t, float2 *sm,
                                           const float2 *__restrict__ tw, const float2 *ptab, Store store) {
  const bool ok0 = bl0 < s.n_blocks, ok1 = bl0 + 1 < s.n_blocks;
  float2 v[16];
  {  // unpack the two blocks through the plan
    const long long bit0 = ok0 ? s.bpar[bl0].src_bit : -1;
    if (bit0 >= 0) {
      // common case: both blocks inside one segment of recorded samples, so
      // sample t + 16 r (r < 32 over the pair) sits at bit p + 16 r * bits of
      // the stream; whole 32-bit words and funnel shifts, no segment walk
      // (the input buffer has spare bytes after the last sample)
      const uint32_t *w = reinterpret_cast<const uint32_t *>(s.src);
      if (s.bits == 2) {
        const int64_t p = bit0 + 2 * t;
        const int64_t w0 = p >> 5;
        const uint32_t sh = (uint32_t)p & 31;
        uint32_t lo = __ldg(w + w0);
#pragma unroll
        for (int r = 0; r < 32; r++) {
          const uint32_t hi = __ldg(w + w0 + r + 1);
          const float x = code_value2(__funnelshift_r(lo, hi, sh) & 3);
          if (r < 16)
            v[r].x = x;
          else
            v[r - 16].y = x;
          lo = hi;
        }
      } else {  // 1-bit: rolled loop through the scratch (small code for the instruction cache)
        float *xs = reinterpret_cast<float *>(sm);
#pragma unroll 1
        for (int r = 0; r < 32; r++) {
          const int64_t p = bit0 + t + 16 * r;
          xs[t + 16 * r] = ((__ldg(w + (p >> 5)) >> (p & 31)) & 1) ? 5.0f : -5.0f;
        }
        pair_from_scratch(v, xs, t);
      }
    } else {  // segment boundaries inside the pair: rare per-sample walk, rolled, through the scratch
      const int o0 = (s.block0 + bl0) * kNd;
      int si = ok0 ? find_segment(s, o0) : 0;
      float *xs = reinterpret_cast<float *>(sm);
#pragma unroll 1
      for (int r = 0; r < 32; r++) xs[t + 16 * r] = (r < 16 ? ok0 : ok1) ? gather_sample(s, o0 + t + 16 * r, si) : 0.0f;
      pair_from_scratch(v, xs, t);
    }
  }
  // The pair's forward transform and the two blocks' inverse ones share one
  // code path (inverse as conj(FFT(conj Y))): h = 0 forward, h = 1, 2 the
  // inverse of block h - 1.  Block 1's ramped half spectrum waits in the
  // scratch behind the transform buffer, ext[16 r + t] for r < 9.
  float2 *ext = sm + kNd + kNd / 16;
  const float4 p0 = ok0 ? s.bpar[bl0].ph : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 p1 = ok1 ? s.bpar[bl0 + 1].ph : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
  for (int h = 0; h < 3; h++) {
    if (h == 2) {
#pragma unroll
      for (int r = 0; r < 9; r++) v[r] = ext[16 * r + t];
#pragma unroll
      for (int r = 9; r < 16; r++) v[r] = make_float2(0.f, 0.f);
    }
    // v[r] = X[t + 16 r]; the transform's reads of sm are complete on return
    // (the inverse inputs are half spectra: v[9..15] == 0)
    fft_reg<-1, 8, false, 15>(v, sm, t, tw, ptab, WarpSync(), h != 0);
    if (h == 0) {
      // split, halve DC/Nyquist, phase ramp; conj of block 0 into v, of block 1 into ext
#pragma unroll
      for (int r = 0; r < 16; r++) sm[padi(t + 16 * r)] = v[r];
      __syncwarp();
      float a_s, a_c, b_s, b_c;
      sincosf(fmaf((float)t, p0.y, p0.x), &a_s, &a_c);
      sincosf(fmaf((float)t, p1.y, p1.x), &b_s, &b_c);
      const float4 st0 = ok0 ? s.bpar[bl0].steps : make_float4(1.f, 0.f, 1.f, 0.f);
      const float4 st1 = ok1 ? s.bpar[bl0 + 1].steps : make_float4(1.f, 0.f, 1.f, 0.f);
      const float as_c = st0.x, as_s = st0.y, bs_c = st1.x, bs_s = st1.y;
#pragma unroll
      for (int r = 0; r < 9; r++) {
        const int k = t + 16 * r;
        float2 f0 = make_float2(0.f, 0.f), f1 = make_float2(0.f, 0.f);
        if (r < 8 || t == 0) {
          const float2 xk = sm[padi(k & (kNd - 1))], xm = sm[padi((kNd - k) & (kNd - 1))];
          const float hf = (k == 0 || k == kNd / 2) ? 0.25f : 0.5f;  // 1/2 of the split, DC and Nyquist halved again
          const float er = hf * (xk.x + xm.x), ei = hf * (xk.y - xm.y);
          const float orr = hf * (xk.y + xm.y), oi = -hf * (xk.x - xm.x);
          // conj(F * (cos phi, -sin phi))
          f0 = make_float2(er * a_c + ei * a_s, er * a_s - ei * a_c);
          f1 = make_float2(orr * b_c + oi * b_s, orr * b_s - oi * b_c);
        }
        v[r] = f0;
        ext[16 * r + t] = f1;
        float c2 = a_c * as_c - a_s * as_s;
        a_s = a_s * as_c + a_c * as_s;
        a_c = c2;
        c2 = b_c * bs_c - b_s * bs_s;
        b_s = b_s * bs_c + b_c * bs_s;
        b_c = c2;
      }
#pragma unroll
      for (int r = 9; r < 16; r++) v[r] = make_float2(0.f, 0.f);
      __syncwarp();  // the split's reads of sm before the next transform writes it
    } else {
      // v = conj(z), z the block's inverse transform: fringe rotation Re(z e^{-i phi}) x amplitude
      const int bl = bl0 + h - 1;
      if (bl < s.n_blocks) {
        const float4 prm = h == 2 ? p1 : p0;
        const float amp = s.bpar[bl].amp;
        const float4 st = s.bpar[bl].steps;
        const float sc = st.z, ss = st.w;
        float rs, rc;
        sincosf(fmaf((float)t, prm.w, prm.z), &rs, &rc);
        rs *= amp;
        rc *= amp;
#pragma unroll
        for (int r = 0; r < 16; r++) {
          store(bl, t + 16 * r, v[r].x * rc - v[r].y * rs);
          const float c2 = rc * sc - rs * ss;
          rs = rs * sc + rc * ss;
          rc = c2;
        }
      }
    }
  }
}

// F-step stage 1 as its own kernel (fringe-stopped samples to s.ts): 16
// pairs of blocks per CTA of 256 threads.
__global__ void __launch_bounds__(256, 4) fstep_block_kernel(const StreamDev *__restrict__ streams,
                                                         const float2 *__restrict__ tw) {
  extern __shared__ __align__(16) float2 sbuf[];  // 16 x kFsScratch
  __shared__ float2 ptab[15 * pass_table_len<8>()];
  const int t = threadIdx.x & 15, grp = threadIdx.x >> 4, warp = threadIdx.x >> 5;
  const StreamDev &s = streams[blockIdx.y];
  float *ts = s.ts;
  fill_pass_table<8, 15>(ptab, tw, threadIdx.x, blockDim.x);
  __syncthreads();
  // 32 blocks per CTA and round, rounds strided over the stream's blocks
  for (int first = blockIdx.x * 32; first < s.n_blocks; first += gridDim.x * 32) {
    if (first + warp * 4 >= s.n_blocks) break;  // whole warps only (warp barriers); later rounds lie further out
    fstep_pair(s, first + grp * 2, t, sbuf + grp * kFsScratch, tw, ptab,
               [ts](int bl, int n, float x) { ts[(int64_t)bl * kNd + n] = x; });
  }
}

// Per-block FP64 parameters of the F-step, one thread per 256-sample block
// (all lanes busy on the reduced-rate FP64 pipe).  Follows
// Delay_correction::do_task / fractional_bit_shift / fringe_stopping
// (sfxc/src/delay_correction.cc:40-47, 97-103, 139-160): the integer and
// fractional delay at the block centre, the fringe phase at the block start
// and its linear step over the block, the amplitude at the centre.  The
// phases leave FP64 only after reduction to one turn.
__device__ __forceinline__ void block_params_one(const StreamDev &s, int bl, int lane);

// CTAs of 128 blocks, strided over the stream's blocks when the grid is
// smaller than the stream (a capped grid leaves room on the SMs to a
// kernel running beside it).
__global__ void __launch_bounds__(128) block_params_kernel(const StreamDev *__restrict__ streams) {
  const StreamDev &s = streams[blockIdx.y];
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * blockDim.x; base < s.n_blocks; base += gridDim.x * blockDim.x) {
    // whole warps stay (neighbour exchange below); lanes past the end compute
    // their block's times (the spline extrapolates) and store nothing
    if (base + (int)(threadIdx.x & ~31) >= s.n_blocks) break;
    block_params_one(s, base + threadIdx.x, lane);
  }
}

__device__ __forceinline__ void block_params_one(const StreamDev &s, int bl, int lane) {
  constexpr double kInvTick = 1.0 / 512000000.0, kInv2Pi = 0.15915494309189533577;
  const int64_t ct = s.start_ticks + (int64_t)(s.block0 + bl) * kNd * s.tps;
  // node intervals: the times grow with the block, so each is walked forward
  // from the launch's first interval (or from the previous time's)
  auto tsec = [&s](int64_t t) { return (double)(t - s.scan_begin) * kInvTick; };
  auto delay = [&s](int64_t t, double v, int i) {
    const double r = spline_eval_at(s.spline, s.spline_n, 0, v, i);
    return s.no_clock ? r : r + (s.clock_offset + (double)(t - s.clock_epoch) * kInvTick * s.clock_rate);
  };
  auto phase = [&s](double v, int i) { return s.phase_zero ? 0.0 : spline_eval_at(s.spline, s.spline_n, 1, v, i); };
  const double v0 = tsec(ct), vc = tsec(ct + s.half_len_ticks);
  const int i0 = spline_walk(s.spline, s.spline_n, v0, s.spline_lo);
  const int ic = spline_walk(s.spline, s.spline_n, vc, i0);
  const double delay_c = delay(ct + s.half_len_ticks, vc, ic);
  const double delay_0 = delay(ct, v0, i0);
  const double phase_0 = phase(v0, i0);
  // the end of a block is the start of the next when a block is a whole
  // number of ticks: take it from the next lane
  const bool chained = s.fft_len_ticks == (int64_t)kNd * s.tps;
  double delay_1 = __shfl_down_sync(0xffffffffu, delay_0, 1);
  double phase_1 = __shfl_down_sync(0xffffffffu, phase_0, 1);
  if (!chained || lane == 31) {
    const double v1 = tsec(ct + s.fft_len_ticks);
    const int i1 = spline_walk(s.spline, s.spline_n, v1, ic);
    delay_1 = delay(ct + s.fft_len_ticks, v1, i1);
    phase_1 = phase(v1, i1);
  }
  if (bl >= s.n_blocks) return;
  const double ampl = s.amp_one ? 1.0 : spline_eval_at(s.spline, s.spline_n, 2, vc, ic);
  const double dis = __dmul_rn(delay_c, (double)s.sample_rate);
  const int integer_delay = (int)floor(__dadd_rn(dis, 0.5));
  // the fractional-delay ramp (phase at bin 0 and step per bin) is stored in
  // FP32 and needs no more: |frac| <= 1/2, the terms stay within a few turns
  const float frac = (float)(dis - integer_delay);
  const float tmp1 = frac * s.frac_scale_f;
  const float tmp2 = (float)(integer_delay & (4 * s.oversamp - 1)) * s.int_phase_q_f;
  const float cterm = tmp2 - tmp1 * s.half_bw_f;
  const float lterm = tmp1 * s.rate_per_bin_f;
  // the fringe phase in FP64 (tens of millions of turns); a zero LO offset or
  // phase model adds exact zeros, skipped
  double phi = s.center_freq * delay_0, phi_end = s.center_freq * delay_1;
  if (s.lo_offset != 0.0) {
    const double lo_phase = s.start_phase + s.lo_offset * ((double)(ct - s.start_ticks) * kInvTick);
    phi = phi + lo_phase;
    phi_end = phi_end + lo_phase + s.fft_len_sec * s.lo_offset;
  } else {
    phi = phi + s.start_phase;
    phi_end = phi_end + s.start_phase;
  }
  if (!s.phase_zero) {
    phi = phi + phase_0 * kInv2Pi;
    phi_end = phi_end + phase_1 * kInv2Pi;
  }
  const double floor_phi = floor(phi);
  phi = s.fringe_mult * (phi - floor_phi);
  phi_end = s.fringe_mult * (phi_end - floor_phi);
  BlockPar bp;
  bp.ph = make_float4(cterm - 6.28318548f * floorf(cterm * 0.159154937f), lterm, (float)phi,
                      (float)((phi_end - phi) * (1.0 / kNd)));
  sincosf(16.0f * bp.ph.y, &bp.steps.y, &bp.steps.x);
  sincosf(16.0f * bp.ph.w, &bp.steps.w, &bp.steps.z);
  bp.amp = (float)ampl;
  bp.pad = 0;
  // unpack source of the pair (bl, bl + 1) when both lie in one recorded segment
  const int o0 = (s.block0 + bl) * kNd;
  const DevSegment sg = s.segs[find_segment(s, o0)];
  bp.src_bit = (bl + 1 < s.n_blocks && sg.src_bit >= 0 && o0 >= sg.out0 && o0 + 2 * kNd <= sg.out0 + sg.n)
                   ? sg.src_bit + (long long)(o0 - sg.out0) * s.bits
                   : -1;
  s.bpar[bl] = bp;
}

// Unpacked samples only (inspection of the Bit2float_worker output).
__global__ void unpack_kernel(const StreamDev *__restrict__ streams, float *__restrict__ out) {
  const StreamDev &s = streams[blockIdx.y];
  const int o0 = (s.block0 + blockIdx.x) * kNd;
  if ((int)blockIdx.x >= s.n_blocks) return;
  int si = find_segment(s, o0 + threadIdx.x);
  out[(int64_t)blockIdx.x * kNd + threadIdx.x] = gather_sample(s, o0 + threadIdx.x, si);
}

// Channel extraction: output byte `ob` of subband s packs spb = 8/fan_out
// samples (extract_byte); sample j reads word ob*spb+j.
__global__ void extract_kernel(const uint8_t *__restrict__ in, int64_t nout, int N, int bits, int fan_out,
                               const int *__restrict__ tracks, uint8_t *__restrict__ out) {
  const int64_t ob = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int sb = blockIdx.y;
  if (ob >= nout) return;
  out[(int64_t)sb * nout + ob] = extract_byte(in + ob * (8 / fan_out) * N, N, bits, fan_out, tracks + sb * fan_out);
}

// ------------------------------------------------------------------------
// F-step, stage 2: windowed real FFT of rot = 2N samples per output row as an
// N-point complex FFT (N = 2^LOGN) of (x[2e], x[2e+1]) by T = N/16 threads,
// then the real-FFT split and the channel selection.  For the tensor-core
// layout ([row][channel][32 stream slots] x 8 B) one thread writes up to four
// streams of a channel as one contiguous piece (a whole 32-byte sector for
// four streams).

// FP16 hi = fp16(s x), lo = fp16(s x - hi) of a complex value (packed
// conversions); SCALE false: x already carries the scale s.
template <bool SCALE>
__device__ __forceinline__ uint2 tc_split(float2 f, float tc_scale) {
  const float2 sv = SCALE ? make_float2(f.x * tc_scale, f.y * tc_scale) : f;
  const __half2 h = __float22half2_rn(sv);
  const float2 hb = __half22float2(h);
  const __half2 l = __float22half2_rn(make_float2(sv.x - hb.x, sv.y - hb.y));
  return make_uint2(*reinterpret_cast<const unsigned *>(&h), *reinterpret_cast<const unsigned *>(&l));
}

// Channel i of one transform Z (natural order, padded): the real-FFT split
// for output bin q = output_offset + i - temp_fft_offset (zero outside 0..N).
// HALF: the split's factor 1/2 applied here; else the transform's input
// carried it (the shared window is scaled by 1/2, which is exact).
template <int N, bool HALF>
__device__ __forceinline__ float2 real_bin(const float2 *Z, const float2 *__restrict__ tw_rot, int q) {
  if (q < 0 || q > N) return make_float2(0.f, 0.f);
  const float2 zk = Z[padi(q & (N - 1))];
  const float2 zc = Z[padi((N - q) & (N - 1))];
  constexpr float h = HALF ? 0.5f : 1.0f;
  const float er = h * (zk.x + zc.x), ei = h * (zk.y - zc.y);
  const float orr = h * (zk.y + zc.y), oi = -h * (zk.x - zc.x);
  const float2 w = __ldg(tw_rot + q);  // q <= N < rot
  return make_float2(er + (orr * w.x - oi * w.y), ei + (orr * w.y + oi * w.x));
}

// Bins q and N - q of one transform together (0 <= q <= N/2): both read
// Z[q] and Z[N - q], and with E, O the even and odd parts and w = tw_rot[q],
// X[q] = E + O w and X[N - q] = conj(E - O w) (tw_rot[N - q] = -conj w).
template <int N, bool HALF>
__device__ __forceinline__ void real_bin_pair(const float2 *Z, float2 w, int q, float2 &xq, float2 &xnq) {
  const float2 zk = Z[padi(q & (N - 1))];
  const float2 zc = Z[padi((N - q) & (N - 1))];
  constexpr float h = HALF ? 0.5f : 1.0f;
  const float er = h * (zk.x + zc.x), ei = h * (zk.y - zc.y);
  const float orr = h * (zk.y + zc.y), oi = -h * (zk.x - zc.x);
  const float owr = orr * w.x - oi * w.y, owi = orr * w.y + oi * w.x;
  xq = make_float2(er + owr, ei + owi);
  xnq = make_float2(er - owr, owi - ei);
}

// First-pass inputs, in two steps so that the loads of the next row can be in
// flight while the current row is written out: raw samples v[qq] = (x[2e],
// x[2e+1]) of complex element e = t + qq T (zero from nper on, or when !ok),
// then the window and, for a sideband flip, the negated odd samples.
// FULL: nper = 2N (every window but NONE), no per-element bounds.
template <int T, bool FULL>
__device__ __forceinline__ void window_raw(float2 (&v)[16], int t, bool ok, int nper, const float *ts) {
  if constexpr (FULL) {
    if (ok) {
#pragma unroll
      for (int qq = 0; qq < 16; qq++) v[qq] = *reinterpret_cast<const float2 *>(ts + 2 * (t + qq * T));
    } else {
#pragma unroll
      for (int qq = 0; qq < 16; qq++) v[qq] = make_float2(0.f, 0.f);
    }
  } else {
#pragma unroll
    for (int qq = 0; qq < 16; qq++) {
      const int i = 2 * (t + qq * T);
      float2 x = make_float2(0.f, 0.f);
      if (ok && i + 1 < nper)
        x = *reinterpret_cast<const float2 *>(ts + i);
      else if (ok && i < nper)
        x.x = ts[i];
      v[qq] = x;
    }
  }
}
// The window is in shared memory (WSMEM) or read through the read-only cache.
// FULL as for window_raw; FLIP: negate the odd samples.
template <int T, bool WSMEM, bool FULL, bool FLIP>
__device__ __forceinline__ void window_apply(float2 (&v)[16], int t, int nper, const float *window) {
  if constexpr (FULL) {
#pragma unroll
    for (int qq = 0; qq < 16; qq++) {
      const int i = 2 * (t + qq * T);
      const float2 w = WSMEM ? *reinterpret_cast<const float2 *>(window + i)
                             : __ldg(reinterpret_cast<const float2 *>(window + i));
      v[qq] = make_float2(v[qq].x * w.x, FLIP ? -(v[qq].y * w.y) : v[qq].y * w.y);
    }
  } else {
    const float sgn = FLIP ? -1.0f : 1.0f;
#pragma unroll
    for (int qq = 0; qq < 16; qq++) {
      const int i = 2 * (t + qq * T);
      if (i + 1 < nper) {
        const float2 w = WSMEM ? *reinterpret_cast<const float2 *>(window + i)
                               : __ldg(reinterpret_cast<const float2 *>(window + i));
        v[qq] = make_float2(v[qq].x * w.x, sgn * (v[qq].y * w.y));
      } else if (i < nper) {
        v[qq] = make_float2(v[qq].x * (WSMEM ? window[i] : __ldg(window + i)), 0.f);
      }
    }
  }
}

// Output row `row` of the NV <= NS streams of a CTA, whose transforms are at
// Z + j * BUF; each goes to its slot in the spectra layout.  sinfo[j] =
// (channel shift output_offset - temp_fft_offset, slot), staged once per CTA.
// `fast`: four (or NS) streams with no shift in consecutive slots from a
// multiple of four, M == N.  Threads tid = 0..nthr-1 share the channels 0..M;
// bins q and N - q come together, so the N/2 + 1 pairs spread evenly (bin N/2
// goes to the last threads on its own).  SCALE: the window was not the
// pre-scaled shared copy, so the split's 1/2 and the tensor-core scale are
// applied here.
template <int N, int NS, int OUT_TC, bool SCALE>
__device__ __forceinline__ void store_row(const float2 *Z, int BUF, const int2 *sinfo, int NV, bool fast, int row,
                                          int nrows_total, int M, int kpad, const float2 *__restrict__ tw_rot,
                                          void *__restrict__ spec_out, float tc_scale, int tid, int nthr) {
  constexpr int S = OUT_TC;  // slots of the tensor-core layout (0: FP32 layout)
  static_assert(NS <= 4, "at most four streams per CTA");
  if constexpr (OUT_TC != 0) {
    constexpr int W = NS;  // streams per store
    uint2 *dst = reinterpret_cast<uint2 *>(spec_out);
    if (fast) {
      auto put = [](uint2 *p, const uint2 (&o)[W]) {
        if constexpr (W == 1) {
          *p = o[0];
        } else if constexpr (W == 2) {
          *reinterpret_cast<uint4 *>(p) = make_uint4(o[0].x, o[0].y, o[1].x, o[1].y);
        } else if constexpr (W == 4) {
          asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "r"(o[0].x), "r"(o[0].y),
                       "r"(o[1].x), "r"(o[1].y), "r"(o[2].x), "r"(o[2].y), "r"(o[3].x), "r"(o[3].y)
                       : "memory");
        } else {
#pragma unroll
          for (int j = 0; j < W; j++) p[j] = o[j];
        }
      };
      const int s0 = sinfo[0].y;
      uint2 *drow = dst + tc_index(row, kpad, 0, s0, S);  // channel i at drow + (i >> 2) * 4S + (i & 3) * 4
      const int gs = 4 * S;
      for (int i = tid; i < N / 2; i += nthr) {
        const float2 w = __ldg(tw_rot + i);
        uint2 a[W], b[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
          float2 xq, xnq;
          real_bin_pair<N, SCALE>(Z + j * BUF, w, i, xq, xnq);
          a[j] = tc_split<SCALE>(xq, tc_scale);
          b[j] = tc_split<SCALE>(xnq, tc_scale);
        }
        put(drow + (i >> 2) * gs + (i & 3) * 4, a);
        put(drow + ((N - i) >> 2) * gs + ((N - i) & 3) * 4, b);
      }
      if (tid >= nthr - W) {  // bin N/2, one stream per thread
        const int j = tid - (nthr - W);
        float2 xq, xnq;
        real_bin_pair<N, SCALE>(Z + j * BUF, __ldg(tw_rot + N / 2), N / 2, xq, xnq);
        dst[tc_index(row, kpad, N / 2, s0 + j, S)] = tc_split<SCALE>(xq, tc_scale);
      }
      return;
    }
    // shifted channels or scattered slots: one 8-byte store per stream and channel
    for (int i = tid; i <= M; i += nthr)
#pragma unroll
      for (int j = 0; j < NS; j++)
        if (j < NV)
          dst[tc_index(row, kpad, i, sinfo[j].y, S)] =
              tc_split<SCALE>(real_bin<N, SCALE>(Z + j * BUF, tw_rot, sinfo[j].x + i), tc_scale);
  } else {
#pragma unroll 1
    for (int j = 0; j < NV; j++) {
      const int shift = sinfo[j].x;
      float2 *dst = reinterpret_cast<float2 *>(spec_out) + ((int64_t)sinfo[j].y * nrows_total + row) * kpad;
      if (shift == 0 && M == N) {
        for (int i = tid; i < N / 2; i += nthr) {
          float2 xq, xnq;
          real_bin_pair<N, SCALE>(Z + j * BUF, __ldg(tw_rot + i), i, xq, xnq);
          dst[i] = xq;
          dst[N - i] = xnq;
        }
        if (tid == nthr - 1 - j) {
          float2 xq, xnq;
          real_bin_pair<N, SCALE>(Z + j * BUF, __ldg(tw_rot + N / 2), N / 2, xq, xnq);
          dst[N / 2] = xq;
        }
      } else {
        for (int i = tid; i <= M; i += nthr) dst[i] = real_bin<N, SCALE>(Z + j * BUF, tw_rot, shift + i);
      }
    }
  }
}

// Stage 2 as its own kernel, reading the fringe-stopped samples from s.ts:
// a CTA of SPC x RPC groups of T threads transforms SPC streams x RPC rows per
// step and steps through a run of rows; the next step's samples are loaded
// into the FFT registers before the current step is written out, so those
// HBM loads overlap the output stores.
template <int LOGN, int SPCMAX = 4>
struct WinShape {
  static constexpr int N = 1 << LOGN, T = N / 16;
  static constexpr int SPC = T * SPCMAX <= 1024 ? SPCMAX : 1024 / T;  // streams per CTA
  static constexpr int RPC = T < 256 ? 256 / T : 1;                   // rows per step
  static constexpr int THREADS = SPC * RPC * T;
  static constexpr int BUF = N + N / 16;  // padded FFT buffer (float2) of one group
  static constexpr size_t FFT_SMEM = (size_t)SPC * RPC * BUF * sizeof(float2);
  // pass-twiddle table of the first eight twiddles per entry (17 KB at
  // N = 4096): the shared memory still fits the same L1 carve-out as the
  // 4-twiddle table, with four fewer complex products per pass (3 % faster);
  // a 15-twiddle table measured 5 % slower than the 4-twiddle one, taking L1
  // capacity from the twice-read input rows
  static constexpr int TWK = 8;
  static constexpr size_t PTB = pass_table_bytes<LOGN, TWK>();
  // the window (up to rot = 2N floats) joins the shared tables when it fits
  static constexpr bool WSMEM = FFT_SMEM + PTB + 8 * N <= 227 * 1024;
  static constexpr size_t SMEM = FFT_SMEM + PTB + (WSMEM ? 8 * N : 0);
  static_assert(THREADS <= 1024, "at most 1024 threads");
};

// OUT_TC: 0 writes the FP32 layout, 32 or 64 the tensor-core layout with that many slots
template <int LOGN, int OUT_TC, int SPCMAX>
__global__ void __launch_bounds__(WinShape<LOGN, SPCMAX>::THREADS, 1024 / WinShape<LOGN, SPCMAX>::THREADS)
    window_fft_kernel(
    const StreamDev *__restrict__ streams, int nstreams, int row0, int nrows, int nrows_total, int steps_per_cta,
    const float *__restrict__ window, const float2 *__restrict__ tw_rot, int nper, int M, int kpad,
    void *__restrict__ spec_out, float tc_scale) {
  using S = WinShape<LOGN, SPCMAX>;
  constexpr int N = S::N, T = S::T, SPC = S::SPC, RPC = S::RPC;
  extern __shared__ __align__(16) float2 dsm[];
  const int t = threadIdx.x % T, g = threadIdx.x / T;
  const int nsg = (nstreams + SPC - 1) / SPC;
  const int sg = blockIdx.x % nsg;  // stream group fastest
  const int nsteps = (nrows + RPC - 1) / RPC;
  const int k0 = (blockIdx.x / nsg) * steps_per_cta, k1 = min(nsteps, k0 + steps_per_cta);
  const int stream = sg * SPC + g % SPC;
  const bool sok = stream < nstreams;
  const StreamDev &s = streams[sok ? stream : 0];
  const bool flip = s.flip != 0;
  // every window but NONE covers the whole transform input: no bounds per element
  const bool full = nper == 2 * N;
  auto row_of = [&](int k) { return k * RPC + g / SPC; };
  auto load_row = [&](float2(&v)[16], int k) {
    const bool ok = sok && row_of(k) < nrows;
    const float *src = s.ts + (int64_t)(row0 + row_of(k)) * N;
    if (full)
      window_raw<T, true>(v, t, ok, nper, src);
    else
      window_raw<T, false>(v, t, ok, nper, src);
  };
  float2 v[16];
  if (k0 < k1) load_row(v, k0);
  // shared tables behind the FFT buffers: pass twiddles, then the window
  float2 *ptab = dsm + S::FFT_SMEM / sizeof(float2);
  fill_pass_table<LOGN, S::TWK>(ptab, tw_rot + 2 * N, threadIdx.x, S::THREADS);
  // the CTA's streams: channel shift and slot, and whether the whole-sector path applies
  __shared__ int2 sinfo[SPC];
  if (threadIdx.x < SPC) {
    const int st = sg * SPC + threadIdx.x;
    sinfo[threadIdx.x] = st < nstreams
                             ? make_int2(streams[st].output_offset - streams[st].temp_fft_offset, streams[st].slot)
                             : make_int2(0, -1);
  }
  // a shared window carries the tensor-core layout's power-of-two scale and
  // the real-FFT split's factor 1/2 (both exact), so the output split needs
  // neither multiply
  const float *win = window;
  if constexpr (S::WSMEM) {
    float4 *wsm = reinterpret_cast<float4 *>(ptab + S::PTB / sizeof(float2));  // nper: a multiple of 4 (rot >= 512)
    const float ws = (OUT_TC ? tc_scale : 1.0f) * 0.5f;
    for (int i = threadIdx.x; i < nper / 4; i += S::THREADS) {
      const float4 w = __ldg(reinterpret_cast<const float4 *>(window) + i);
      wsm[i] = make_float4(w.x * ws, w.y * ws, w.z * ws, w.w * ws);
    }
    win = reinterpret_cast<const float *>(wsm);
  }
  __syncthreads();
  const int nv = min(SPC, nstreams - sg * SPC);
  bool fast = OUT_TC && M == N && nv == SPC && sinfo[0].y % SPC == 0;
#pragma unroll
  for (int j = 0; j < SPC; j++) fast = fast && sinfo[j].x == 0 && sinfo[j].y == sinfo[0].y + j;
#pragma unroll 1
  for (int k = k0; k < k1; k++) {
    if (full) {
      if (flip)
        window_apply<T, S::WSMEM, true, true>(v, t, nper, win);
      else
        window_apply<T, S::WSMEM, true, false>(v, t, nper, win);
    } else {
      if (flip)
        window_apply<T, S::WSMEM, false, true>(v, t, nper, win);
      else
        window_apply<T, S::WSMEM, false, false>(v, t, nper, win);
    }
    // tw_rot holds exp(-2 pi i m / rot) for m < rot, followed by exp(-2 pi i m / N) for m < N.
    // Each group's transform synchronises only its own T threads (named
    // barrier 1 + g) when the groups are whole warps and few enough.
    // FP32 layout: each group writes its own stream's row (whole lines), so
    // the groups synchronise only themselves and run out of step with each
    // other (18 % faster at 4096 channels than the CTA-wide barriers the
    // tensor-core layout's shared 32-byte pieces need)
    constexpr bool kIndep = OUT_TC == 0 && T >= 32 && S::THREADS / T <= 15;
    if constexpr (kIndep) {
      const GroupSync gs{1 + g, T};
      fft_reg<-1, LOGN, true, S::TWK>(v, dsm + g * S::BUF, t, tw_rot + 2 * N, ptab, gs);
      gs();
      if (k + 1 < k1) load_row(v, k + 1);
      const int j = g % SPC, row = row_of(k);
      if (j < nv && row < nrows) {
        const float2 *Z = dsm + g * S::BUF;
        const int shift = sinfo[j].x;
        float2 *dst = reinterpret_cast<float2 *>(spec_out) + ((int64_t)sinfo[j].y * nrows_total + row0 + row) * kpad;
        if (shift == 0 && M == N) {
          for (int i = t; i < N / 2; i += T) {
            float2 xq, xnq;
            real_bin_pair<N, !S::WSMEM>(Z, __ldg(tw_rot + i), i, xq, xnq);
            dst[i] = xq;
            dst[N - i] = xnq;
          }
          if (t == T - 1) {
            float2 xq, xnq;
            real_bin_pair<N, !S::WSMEM>(Z, __ldg(tw_rot + N / 2), N / 2, xq, xnq);
            dst[N / 2] = xq;
          }
        } else {
          for (int i = t; i <= M; i += T) dst[i] = real_bin<N, !S::WSMEM>(Z, tw_rot, shift + i);
        }
      }
      gs();  // the next step's transform rewrites the group's buffer
      continue;
    }
    if constexpr (T >= 32 && S::THREADS / T <= 15) {
      fft_reg<-1, LOGN, true, S::TWK>(v, dsm + g * S::BUF, t, tw_rot + 2 * N, ptab, GroupSync{1 + g, T});
      __syncthreads();  // the stores read every group's transform
    } else {
      fft_reg<-1, LOGN, true, S::TWK>(v, dsm + g * S::BUF, t, tw_rot + 2 * N, ptab, BlockSync());
    }
    if (k + 1 < k1) load_row(v, k + 1);  // hop = rot / 2
#pragma unroll 1
    for (int r = 0; r < RPC; r++) {
      const int row = k * RPC + r;
      if (row >= nrows) break;
      store_row<N, SPC, OUT_TC, !S::WSMEM>(dsm + r * SPC * S::BUF, S::BUF, sinfo, nv, fast, row0 + row, nrows_total,
                                           M, kpad, tw_rot, spec_out, tc_scale, threadIdx.x, S::THREADS);
    }
    // the next step's FFT rewrites the buffers (placing this barrier inside
    // that FFT, after its first radix-16 pass, measured 1.7 % slower)
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// Bit statistics.
// Code counts of 8 bits (mask 0x55) or 32 bits (mask 0x55555555): 2-bit
// codes -> c[code] with code = 2 * high bit + low bit; 1-bit -> c[bit value].
__device__ __forceinline__ void count_codes(uint32_t x, int nbits, int bits, uint32_t (&c)[4]) {
  if (bits == 2) {
    const uint32_t m = nbits == 32 ? 0x55555555u : 0x55u;
    const uint32_t lo = x & m, hi = (x >> 1) & m;
    c[3] = __popc(hi & lo);
    c[2] = __popc(hi & ~lo & m);
    c[1] = __popc(~hi & lo & m);
    c[0] = nbits / 2 - c[1] - c[2] - c[3];
  } else {
    c[1] = __popc(nbits == 32 ? x : x & 0xFFu);
    c[0] = nbits - c[1];
    c[2] = c[3] = 0;
  }
}

// Cal-diode state over increasing counted-byte indices: toggles at t0,
// t0 + period, ... (once when period <= 0, never when t0 <= 0).  at() places
// the walker with one division, advance() steps it forward without any.
struct CalWalk {
  int on;
  int64_t next, period;
  __device__ __forceinline__ void at(const StreamDev &s, int64_t c) {
    on = 1;
    next = INT64_MAX;
    period = s.tsys_period;
    if (s.tsys_two_bit) {
      on = s.tsys_on0;
      if (s.tsys_t0 > 0) {
        if (c >= s.tsys_t0) {
          const int64_t flips = period > 0 ? 1 + (c - s.tsys_t0) / period : 1;
          on ^= (int)(flips & 1);
          next = period > 0 ? s.tsys_t0 + flips * period : INT64_MAX;
        } else {
          next = s.tsys_t0;
        }
      }
    }
  }
  __device__ __forceinline__ void advance(int64_t c) {
    while (c >= next) {
      on ^= 1;
      next = period > 0 ? next + period : INT64_MAX;
    }
  }
};

struct CodeCounts {
  uint32_t on[4], off[4];
  __device__ __forceinline__ void add(uint32_t x, int nbits, int bits, int cal_on) {
    uint32_t c[4];
    count_codes(x, nbits, bits, c);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      on[k] += cal_on ? c[k] : 0u;
      off[k] += cal_on ? 0u : c[k];
    }
  }
};

// Code counts of the counted bytes src[0, n) (counted index cfirst + j for
// src[j]) by a group of NL threads: bytes before the first 16-byte boundary
// and after the last one singly, the middle as 16-byte loads (four in flight
// per thread) counted a word at a time unless a cal-diode toggle falls
// inside the word.
template <int NL>
__device__ __forceinline__ void count_span(const StreamDev &s, const uint8_t *src, int n, int64_t cfirst, int lane,
                                           CodeCounts &cc) {
  const int bits = s.bits;
  const int head = min(n, (int)((16 - ((uintptr_t)src & 15)) & 15));
  const int nvec = (n - head) / 16;
  const int tail0 = head + 16 * nvec;
  for (int j = lane; j < head + (n - tail0); j += NL) {
    const int pos = j < head ? j : tail0 + (j - head);
    CalWalk w;
    w.at(s, cfirst + pos);
    cc.add(__ldg(src + pos), 8, bits, w.on);
  }
  if (lane >= nvec) return;
  const uint4 *vsrc = reinterpret_cast<const uint4 *>(src + head);
  const int64_t cvec = cfirst + head;
  CalWalk w;
  w.at(s, cvec + 16 * (int64_t)lane);
  for (int q0 = lane; q0 < nvec; q0 += 4 * NL) {
    uint4 v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int q = q0 + u * NL;
      v[u] = q < nvec ? __ldg(vsrc + q) : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int q = q0 + u * NL;
      if (q >= nvec) break;
      const int64_t c0 = cvec + 16 * (int64_t)q;
      w.advance(c0);
      const uint32_t ww[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
      if (c0 + 16 <= w.next) {
#pragma unroll
        for (int k = 0; k < 4; k++) cc.add(ww[k], 32, bits, w.on);
      } else {
        for (int b = 0; b < 16; b++) {
          w.advance(c0 + b);
          cc.add((ww[b >> 2] >> (8 * (b & 3))) & 0xFFu, 8, bits, w.on);
        }
      }
    }
  }
}

// Bit statistics over the counted-byte ranges, as per-code counts split by
// the cal-diode state: s.hist[0..3] on, [4..7] off (the byte histogram of
// bit_statistics.cc:36-47 enters the levels and tsys values only through
// these counts).  Work items (stream, first range, range count, offset):
// range count > 0 packs that many short ranges, one warp per range; range
// count 0 is the 64 KB piece at `offset` of one long range, all warps.
__global__ void __launch_bounds__(256) bitstat_kernel(const StreamDev *__restrict__ streams,
                                                     const int4 *__restrict__ items, int nitems) {
  const int4 it = items[blockIdx.x];
  const StreamDev &s = streams[it.x];
  CodeCounts cc = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (it.z > 0) {
    for (int r = it.y + warp; r < it.y + it.z; r += blockDim.x >> 5) {
      const DevStatRange rg = s.stats[r];
      count_span<32>(s, s.src + rg.src_byte, rg.n, rg.cidx, lane, cc);
    }
  } else {
    const DevStatRange rg = s.stats[it.y];
    const int n = min(65536, rg.n - it.w);
    count_span<256>(s, s.src + rg.src_byte + it.w, n, (int64_t)rg.cidx + it.w, threadIdx.x, cc);
  }
  // warp sums, one global update per counter and warp
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint32_t a = cc.on[k], b = cc.off[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      if (a) atomicAdd(&s.hist[k], (unsigned long long)a);
      if (b) atomicAdd(&s.hist[4 + k], (unsigned long long)b);
    }
  }
}

// ------------------------------------------------------------------------
// X-step on CUDA cores (Correlation_core::integration_step,
// sfxc/src/correlation_core.cc:241-273; binned: Correlation_core_pulsar::
// integration_step, sfxc/src/correlation_core_pulsar.cc:101-146).
// spec: [stream][row][kpad] complex64.  Work items -- (32-channel tile, block
// of rows, part of the stream-pair tiles) -- are dealt to persistent CTAs.  A
// CTA stages R rows x npad streams x 32 channels per step through a 4-deep
// cp.async ring (one barrier per R rows), so the loads of three steps are in
// flight while one is multiplied; each thread owns one channel and up to TPW
// tiles of 4x4 stream pairs (i in tile row I, j in tile column J, I <= J) in
// registers, and adds them to the accumulators with float2 atomics when its
// item ends, or, binned, when its channel's pulsar bin changes (acc[bin]).
// blmap[i*npad+j] gives (baseline << 1 | conj) or -1.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

template <int TPW, bool BINNED>
__global__ void __launch_bounds__(384, 1) xcorr_f32_kernel(const __grid_constant__ F32Args a) {
  extern __shared__ __align__(16) float2 xs[];  // kF32Stages x [R rows][npad streams][32 channels]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nct = (a.K + 31) / 32;
  const int nrows = a.r1 - a.r0;
  const int nrb = (nrows + a.rblock - 1) / a.rblock;
  const int nitems = nct * nrb * a.nparts;
  const int stage_f2 = a.R * a.npad * 32;  // float2 per stage
  const int chunks = a.R * a.npad * 16;    // 16-byte copies per stage
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int part = item % a.nparts, rb = (item / a.nparts) % nrb, ct = item / (a.nparts * nrb);
    const int k = ct * 32 + lane;
    const int ra = a.r0 + rb * a.rblock, rz = min(a.r1, ra + a.rblock);
    const int t_end = min(a.ntiles, (part + 1) * a.tiles_per_part);
    int ti[TPW], tj[TPW];
    float2 v[TPW][4][4];
#pragma unroll
    for (int t = 0; t < TPW; t++) {
      const int tile = part * a.tiles_per_part + warp + t * nwarps;
      ti[t] = tile < t_end ? a.tiles[2 * tile] : -1;
      tj[t] = tile < t_end ? a.tiles[2 * tile + 1] : -1;
#pragma unroll
      for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) v[t][p][q] = make_float2(0.f, 0.f);
    }
    // add the register tiles to acc[bin] (bin 0 when not binned), or store
    // them as this row block's partial sums (a.part), and clear them.  Each
    // (bin, baseline, channel) entry has one writer thread per launch (or per
    // row block with partial sums), so the results do not depend on timing.
    auto flush = [&](int bin) {
      if (k >= a.K || bin < 0) return;
#pragma unroll
      for (int t = 0; t < TPW; t++) {
        if (ti[t] < 0) continue;
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const int m = __ldg(a.blmap + (ti[t] * 4 + p) * a.npad + tj[t] * 4 + q);
            if (m >= 0) {
              const float2 x = v[t][p][q];
              const float2 y = make_float2(x.x, (m & 1) ? -x.y : x.y);
              if (a.part) {
                a.part[((int64_t)rb * a.nbl + (m >> 1)) * a.kpad + k] = y;
              } else {
                // the entry's only writer in this launch: its adds land in
                // program order, so the sum does not depend on timing; the
                // atomic lets the thread go on without waiting for the load
                atomicAdd(a.acc + ((int64_t)bin * a.nbl + (m >> 1)) * a.kpad + k, y);
              }
            }
            v[t][p][q] = make_float2(0.f, 0.f);
          }
      }
    };
    const int nsteps = (rz - ra + a.R - 1) / a.R;
    auto issue = [&](int step) {
      if (step < nsteps) {
        float2 *dst = xs + (step % kF32Stages) * stage_f2;
        const int rs = ra + step * a.R;
        for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
          const int rr = c / (a.npad * 16), rem = c - rr * (a.npad * 16), st = rem >> 4, cc = (rem & 15) * 2;
          const int row = rs + rr, kk = ct * 32 + cc;
          // channel kk + 1 may be K, which lies inside the padded row (kpad >= K + 3)
          const bool ok = row < rz && st < a.nstreams && kk < a.K;
          const float2 *src = ok ? a.spec + ((int64_t)st * a.nrows_total + row) * a.kpad + kk : a.spec;
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst + (rr * a.npad + st) * 32 + cc)),
                       "l"(src), "r"(ok ? 16 : 0)
                       : "memory");
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");  // possibly empty: keeps the group count per step
    };
#pragma unroll 1
    for (int s = 0; s < kF32Stages - 1; s++) issue(s);
    int cur = -1;
#pragma unroll 1
    for (int step = 0; step < nsteps; step++) {
      asm volatile("cp.async.wait_group %0;" ::"n"(kF32Stages - 2) : "memory");
      __syncthreads();  // step's rows are in; every thread is done with the slot refilled next
      issue(step + kF32Stages - 1);
      const float2 *xst = xs + (step % kF32Stages) * stage_f2;
#pragma unroll 1
      for (int rr = 0; rr < a.R; rr++) {
        const int row = ra + step * a.R + rr;
        if (row >= rz) break;
        if constexpr (BINNED) {
          const int bin = k < a.K ? __ldg(a.bins + (int64_t)k * a.bins_rows + (row - a.r0)) : -1;
          if (bin != cur) {
            flush(cur);
            cur = bin;
          }
        }
        const float2 *xr = xst + rr * a.npad * 32 + lane;
#pragma unroll
        for (int t = 0; t < TPW; t++) {
          if (ti[t] < 0) continue;
          float2 xi[4], xj[4];
#pragma unroll
          for (int p = 0; p < 4; p++) {
            xi[p] = xr[(ti[t] * 4 + p) * 32];
            xj[p] = xr[(tj[t] * 4 + p) * 32];
          }
#pragma unroll
          for (int p = 0; p < 4; p++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
              // x_i * conj(x_j)
              v[t][p][q].x = fmaf(xi[p].x, xj[q].x, fmaf(xi[p].y, xj[q].y, v[t][p][q].x));
              v[t][p][q].y = fmaf(xi[p].y, xj[q].x, fmaf(-xi[p].x, xj[q].y, v[t][p][q].y));
            }
        }
      }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    flush(BINNED ? cur : 0);
    __syncthreads();  // the ring is refilled by the next item
  }
}

// Partial sums of the row blocks into the accumulators, in row-block order.
__global__ void f32_part_reduce_kernel(const float2 *__restrict__ part, int nrb, int nbl, int kpad, int K,
                                       float2 *__restrict__ acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
  if (k >= K) return;
  float2 s = acc[(int64_t)b * kpad + k];
  for (int r = 0; r < nrb; r++) {
    const float2 x = part[((int64_t)r * nbl + b) * kpad + k];
    s = make_float2(s.x + x.x, s.y + x.y);
  }
  acc[(int64_t)b * kpad + k] = s;
}

// ------------------------------------------------------------------------
// Pulsar bins (Correlation_core_pulsar::dedisperse_buffer) in FP64, evaluated
// with the reference's operation order so that every bin matches; written
// [channel][row] (row fastest) for the per-channel sort and the binned X-steps.
__global__ void pulsar_bins_kernel(int nrows, int K, double start_phase, double rate_term, double fft_duration,
                                   const double *__restrict__ offsets, double g0, double g1, int nbins,
                                   int16_t *__restrict__ bins) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (k >= K || r >= nrows) return;
  const double us_per_day = 86400000000.0;
  // start_phase + (coef[1] + 60 F0) * fft_duration * current_fft * 1440 / us_per_day
  double ph = __dmul_rn(rate_term, fft_duration);
  ph = __dmul_rn(ph, (double)r);
  ph = __dmul_rn(ph, 1440.0);
  ph = __ddiv_rn(ph, us_per_day);
  ph = __dadd_rn(start_phase, ph);
  double p = __dsub_rn(ph, offsets[k]);
  p = __dsub_rn(p, floor(p));
  const double len = __dsub_rn(g1, g0);
  int bin;
  if (p >= g0) {
    bin = p < g1 ? (int)__ddiv_rn(__dmul_rn(__dsub_rn(p, g0), (double)(nbins - 1)), len) + 1 : 0;
  } else if (__dadd_rn(p, 1.0) < g1) {
    bin = (int)__ddiv_rn(__dmul_rn(__dsub_rn(__dadd_rn(p, 1.0), g0), (double)(nbins - 1)), len) + 1;
  } else {
    bin = 0;
  }
  bins[(int64_t)k * nrows + r] = (int16_t)bin;
}

// ------------------------------------------------------------------------
// Normalisation.  norms[i] = max(1, sum_k Re acc[auto_i][k] / M) in FP64.
__global__ void norm_autos_kernel(const float2 *__restrict__ acc, int kpad, int M, int nstreams, double *norms) {
  __shared__ double red[256];
  const int i = blockIdx.x;
  double s = 0.0;
  for (int k = threadIdx.x; k <= M; k += blockDim.x) s += (double)acc[(int64_t)i * kpad + k].x;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double n = red[0] / M;
    norms[i] = n < 1 ? 1 : n;
  }
}

// out[b][k] (compact M+1) = normalised visibility; flagfac[b] = N1*N2 (crosses).
// A cross baseline's FP64 norm is the same for all its channels: one thread
// of the CTA (all of whose threads share the baseline) computes it.
__global__ void normalize_kernel(const float2 *__restrict__ acc, int kpad, int M, int nstreams, int nbl,
                                 const int *__restrict__ bl, const double *__restrict__ norms,
                                 const double *__restrict__ flagfac, float2 *__restrict__ out) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ float cross_norm;
  if (b >= nstreams && threadIdx.x == 0)
    cross_norm = (float)sqrt(flagfac[b] * norms[bl[2 * b]] * norms[bl[2 * b + 1]]);
  __syncthreads();
  if (k > M) return;
  const float2 v = acc[(int64_t)b * kpad + k];
  float2 o;
  if (b < nstreams) {
    o = make_float2((float)((double)v.x / norms[b]), 0.f);
  } else {
    const float norm = cross_norm;
    o = make_float2(v.x / norm, v.y / norm);
  }
  out[(int64_t)b * (M + 1) + k] = o;
}

// ------------------------------------------------------------------------
// Phased array: Correlation_core_phased::integration_step (sfxc/src/
// correlation_core_phased.cc:113-126) -- each FFT's spectra of all streams
// added, in stream order, to the buffer of its sub-integration; one thread
// per channel keeps the running sum of the current buffer in registers.
__global__ void phased_kernel(const float2 *__restrict__ spec, int nrows_total, int kpad, int nstreams, int r0,
                              int nrows, int K, int nsub, float2 *__restrict__ acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K || nrows <= 0) return;
  int s = r0 / nsub;
  float2 sum = acc[(size_t)s * kpad + k];
  for (int r = 0; r < nrows; r++) {
    const int sr = (r0 + r) / nsub;
    if (sr != s) {
      acc[(size_t)s * kpad + k] = sum;
      s = sr;
      sum = acc[(size_t)s * kpad + k];
    }
    for (int i = 0; i < nstreams; i++) {
      const float2 x = spec[((size_t)i * nrows_total + r) * kpad + k];
      sum = make_float2(sum.x + x.x, sum.y + x.y);
    }
  }
  acc[(size_t)s * kpad + k] = sum;
}

// ------------------------------------------------------------------------
// Extra phase centres: Correlation_core::sub_integration (sfxc/src/
// correlation_core.cc:516-559) with uvshift (561-593).  Every channel of
// every baseline of the sub-integration goes to each centre's accumulator;
// a cross baseline of centre c >= 1 first gets the amplitude and the phase
// phi + k delta of its residual delay (FP64 angle, FP32 product, as the
// reference's FP64 recurrence and complex<float> arithmetic).
__global__ void pc_dump_kernel(float2 *__restrict__ acc, float2 *__restrict__ pcacc, const UvShift *__restrict__ uvp,
                               int nstreams, int nbl, int kpad, int K, int npc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
  if (k >= K) return;
  const size_t i = (size_t)b * kpad + k, cstride = (size_t)nbl * kpad;
  const float2 x = acc[i];
  pcacc[i] = make_float2(pcacc[i].x + x.x, pcacc[i].y + x.y);
  for (int c = 1; c < npc; c++) {
    float2 &p = pcacc[c * cstride + i];
    if (b < nstreams) {
      p = make_float2(p.x + x.x, p.y + x.y);
    } else {
      const UvShift u = uvp[(size_t)(c - 1) * nbl + b];
      double sn, cs;
      sincos(fma((double)k, u.delta, u.phi), &sn, &cs);
      const float amp = (float)u.amp, cf = (float)cs, sf = (float)sn;
      const float xr = amp * x.x, xi = amp * x.y;
      p = make_float2(p.x + (xr * cf - xi * sf), p.y + (xr * sf + xi * cf));
    }
  }
  acc[i] = make_float2(0.f, 0.f);
}

// ------------------------------------------------------------------------
// Spectral reduction (number_channels < fft_size_correlation):
// Correlation_core::integration_write, sfxc/src/correlation_core.cc:413-439.
// One CTA per normalised spectrum X[0..M]: optional normalisation to unit
// amplitude, the mask, an unnormalised complex-to-real FFT of 2M points (the
// imaginary parts of DC and Nyquist ignored) as one M-point complex FFT of
// the even and odd lags, the lags folded to 2 nch (lag nch the mean of +-nch),
// the lag window, a real FFT of 2 nch points as one nch-point complex FFT and
// the real split, a division by 2M.  Both transforms are in-place radix-2 in
// shared memory: the work is one spectrum per baseline per integration.

// in-place radix-2 transform of the 2^logn values a[] in bit-reversed order:
// sign -1 forward, +1 backward; twiddles exp(-2 pi i j / len) = tw2M[j 2M / len]
__device__ void smem_fft_radix2(float2 *a, int logn, int sign, const float2 *__restrict__ tw2M, int M) {
  const int n = 1 << logn;
  for (int s = 1; s <= logn; s++) {
    const int len = 1 << s, half = len >> 1, stride = (2 * M) >> s;
    for (int b = threadIdx.x; b < n / 2; b += blockDim.x) {
      const int j = b & (half - 1), i = (b - j) * 2 + j;
      float2 w = __ldg(tw2M + j * stride);
      if (sign > 0) w.y = -w.y;
      const float2 u = a[i], x = a[i + half];
      const float2 v = make_float2(x.x * w.x - x.y * w.y, x.x * w.y + x.y * w.x);
      a[i] = make_float2(u.x + v.x, u.y + v.y);
      a[i + half] = make_float2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) reduce_kernel(const float2 *__restrict__ in, int M, int logM, int nch,
                                                     int lognch, const float *__restrict__ mask,
                                                     const float *__restrict__ lagwin, int normalize,
                                                     const float2 *__restrict__ tw2M, float2 *__restrict__ out) {
  extern __shared__ __align__(16) float2 rsm[];
  float2 *a = rsm;                                   // M complex
  float *lag = reinterpret_cast<float *>(rsm + M);   // 2 nch lags
  const float2 *X = in + (size_t)blockIdx.x * (M + 1);
  auto load = [&](int k) {
    float2 x = X[k];
    if (normalize) {
      const float m = hypotf(x.x, x.y);
      if (m != 0.0f) x = make_float2(x.x / m, x.y / m);
    }
    const float mk = mask[k];
    return make_float2(x.x * mk, x.y * mk);
  };
  // c2r of 2M points: even lags e = IDFT(X[k] + conj X[M-k]), odd lags
  // o = IDFT((X[k] - conj X[M-k]) e^{i pi k / M}); z = e + i o
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    float2 xk = load(k), xm = load(M - k);
    if (k == 0) xk.y = xm.y = 0.0f;
    const float2 e = make_float2(xk.x + xm.x, xk.y - xm.y);
    const float2 d = make_float2(xk.x - xm.x, xk.y + xm.y);
    const float2 w = __ldg(tw2M + k);  // exp(-i pi k / M); d * conj(w)
    const float2 o = make_float2(d.x * w.x + d.y * w.y, d.y * w.x - d.x * w.y);
    a[__brev((unsigned)k) >> (32 - logM)] = make_float2(e.x - o.y, e.y + o.x);
  }
  __syncthreads();
  smem_fft_radix2(a, logM, +1, tw2M, M);
  auto lag_at = [&](int q) { return (q & 1) ? a[q >> 1].y : a[q >> 1].x; };  // r[q], q < 2M
  for (int q = threadIdx.x; q < 2 * nch; q += blockDim.x) {
    float v;
    if (q < nch)
      v = lag_at(q);
    else if (q == nch)
      v = (lag_at(nch) + lag_at(2 * M - nch)) / 2;
    else
      v = lag_at(2 * M - nch + (q - nch));
    lag[q] = v * lagwin[q];
  }
  __syncthreads();
  for (int n = threadIdx.x; n < nch; n += blockDim.x)
    a[__brev((unsigned)n) >> (32 - lognch)] = make_float2(lag[2 * n], lag[2 * n + 1]);
  __syncthreads();
  smem_fft_radix2(a, lognch, -1, tw2M, M);
  // r2c split: A[k] = E + W^k O, W = exp(-2 pi i / 2nch) = tw2M[M / nch]
  float2 *Y = out + (size_t)blockIdx.x * (nch + 1);
  const float scale = (float)(2 * M);
  for (int k = threadIdx.x; k <= nch; k += blockDim.x) {
    const float2 zk = a[k & (nch - 1)], zc = a[(nch - k) & (nch - 1)];
    const float er = 0.5f * (zk.x + zc.x), ei = 0.5f * (zk.y - zc.y);
    const float orr = 0.5f * (zk.y + zc.y), oi = -0.5f * (zk.x - zc.x);
    const float2 w = __ldg(tw2M + (size_t)k * (M / nch));
    Y[k] = make_float2((er + (orr * w.x - oi * w.y)) / scale, (ei + (orr * w.y + oi * w.x)) / scale);
  }
}

// ------------------------------------------------------------------------
// launchers
static int sm_count() {
  static const int n = [] {  // initialised once, also when contexts are planned from several threads
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    return cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 1;
  }();
  return n;
}

void launch_block_params(const StreamDev *d_streams, int nstreams, int max_blocks, cudaStream_t st,
                         int ctas_per_sm) {
  int x = (max_blocks + 127) / 128;
  if (ctas_per_sm > 0) x = std::max(1, std::min(x, ctas_per_sm * sm_count() / nstreams));
  block_params_kernel<<<dim3(x, nstreams), 128, 0, st>>>(d_streams);
}

void launch_fstep_block(const StreamDev *d_streams, int nstreams, int max_blocks, const float2 *tw256,
                        cudaStream_t st) {
  launch_block_params(d_streams, nstreams, max_blocks, st);
  launch_fstep(d_streams, nstreams, max_blocks, tw256, st, 0);
}

void launch_fstep(const StreamDev *d_streams, int nstreams, int max_blocks, const float2 *tw256, cudaStream_t st,
                  int ctas_per_sm) {
  // by default about three waves of 4 resident CTAs per SM, each CTA looping
  // over rounds (measured against 1, 2, 4 and 6 waves on the 32-stream,
  // 4096-channel job: 2 % faster than two, the others slower still); the
  // autotuner may pick another count per shape
  const int per_stream = std::max(1, (ctas_per_sm > 0 ? ctas_per_sm : 12) * sm_count() / nstreams);
  dim3 grid(std::min((max_blocks + 31) / 32, per_stream), nstreams);
  constexpr int smem = 16 * kFsScratch * sizeof(float2);
  cudaFuncSetAttribute(fstep_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  fstep_block_kernel<<<grid, 256, smem, st>>>(d_streams, tw256);
}

void launch_unpack(const StreamDev *d_streams, int nstreams, int max_blocks, float *out, cudaStream_t st) {
  unpack_kernel<<<dim3(max_blocks, nstreams), kNd, 0, st>>>(d_streams, out);
}

void launch_extract(const uint8_t *in, int64_t nout, int N, int bits, int nsub, int fan_out, const int *tracks,
                    uint8_t *out, cudaStream_t st) {
  extract_kernel<<<dim3((unsigned)((nout + 255) / 256), nsub), 256, 0, st>>>(in, nout, N, bits, fan_out, tracks, out);
}

// ------------------------------------------------------------- phase cal ---
// Phase-cal folding (Input_node_data_writer::do_phasecal,
// sfxc/src/input_node_data_writer.cc:230-312): byte j of run r, data[off + j],
// holds the samples of bins ((bin0 + j) mod pb) * spb + q, q < spb = 8 / bits,
// LSB first, and they go to accumulator row r.row (pb * spb int32 bins).
// Thread t takes every pb-th byte of the run, those of byte-bin t, so that a
// warp reads consecutive bytes, and adds its spb sums once: integer sums, so
// neither the order nor the atomics change the result.
template <int BITS>
__global__ void __launch_bounds__(256) phasecal_kernel(const uint8_t *data, const PcalRun *runs, int pb,
                                                       int32_t *acc) {
  constexpr int SPB = 8 / BITS;
  const PcalRun r = runs[blockIdx.y];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= pb) return;
  int j = t - r.bin0;
  if (j < 0) j += pb;
  int sum[SPB] = {};
  for (; j < r.n; j += pb) {
    const uint32_t v = __ldg(data + r.off + j);
#pragma unroll
    for (int q = 0; q < SPB; q++) {
      // Bit2float / do_phasecal sample values: 2-bit {-7, -2, 2, 7}, 1-bit {-5, 5}
      if (BITS == 2)
        sum[q] += (int)(int8_t)(uint8_t)(0x0702FEF9u >> (8 * ((v >> (2 * q)) & 3)));
      else
        sum[q] += ((v >> q) & 1) ? 5 : -5;
    }
  }
  int32_t *a = acc + (int64_t)r.row * pb * SPB + (int64_t)t * SPB;
#pragma unroll
  for (int q = 0; q < SPB; q++)
    if (sum[q]) atomicAdd(a + q, sum[q]);
}

void launch_phasecal(const uint8_t *data, const PcalRun *runs, int nruns, int pb, int bits, int32_t *acc,
                     cudaStream_t st) {
  for (int r0 = 0; r0 < nruns; r0 += 65535) {
    const dim3 grid((unsigned)((pb + 255) / 256), (unsigned)std::min(65535, nruns - r0));
    if (bits == 2)
      phasecal_kernel<2><<<grid, 256, 0, st>>>(data, runs + r0, pb, acc);
    else
      phasecal_kernel<1><<<grid, 256, 0, st>>>(data, runs + r0, pb, acc);
  }
}

template <int LOGN, int OUT_TC, int SPCMAX>
static void window_fft_launch_spc(const StreamDev *d_streams, int nstreams, int row0, int nrows, int nrows_total,
                                  const float *window, const float2 *tw_rot, int nper, int M, int kpad, void *spec,
                                  float tc_scale, cudaStream_t st, int waves) {
  using S = WinShape<LOGN, SPCMAX>;
  const int nsg = (nstreams + S::SPC - 1) / S::SPC, nsteps = (nrows + S::RPC - 1) / S::RPC;
  // runs of steps so that the CTAs fill two waves by default (three or four
  // waves measured 1 % slower on the 32-stream, 4096-channel job); the
  // autotuner may pick another count per shape
  const int per_sm = 1024 / S::THREADS;
  const int runs = std::max(1, std::min(nsteps, (waves > 0 ? waves : 2) * per_sm * sm_count() / nsg));
  const int steps_per_cta = (nsteps + runs - 1) / runs;
  const unsigned grid = (unsigned)(nsg * ((nsteps + steps_per_cta - 1) / steps_per_cta));
  auto kern = window_fft_kernel<LOGN, OUT_TC, SPCMAX>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
  kern<<<grid, S::THREADS, S::SMEM, st>>>(d_streams, nstreams, row0, nrows, nrows_total, steps_per_cta, window, tw_rot,
                                          nper, M, kpad, spec, tc_scale);
}

template <int LOGN, int OUT_TC>
static void window_fft_launch(const StreamDev *d_streams, int nstreams, int row0, int nrows, int nrows_total,
                              const float *window, const float2 *tw_rot, int nper, int M, int kpad, void *spec,
                              float tc_scale, cudaStream_t st, int waves) {
  // four streams per CTA: a whole 32-byte sector per channel in the TC layout
  // (two streams per CTA, two CTAs per SM, measured 20 % slower; each group
  // writing its own stream's 8-byte pieces, without the CTA-wide barriers,
  // 74 % slower)
  window_fft_launch_spc<LOGN, OUT_TC, 4>(d_streams, nstreams, row0, nrows, nrows_total, window, tw_rot, nper, M, kpad,
                                         spec, tc_scale, st, waves);
}

#define SFXC_LOGN_SWITCH(logn, CALL) \
  switch (logn) {                    \
    case 8: CALL(8); break;          \
    case 9: CALL(9); break;          \
    case 10: CALL(10); break;        \
    case 11: CALL(11); break;        \
    case 12: CALL(12); break;        \
    case 13: CALL(13); break;        \
    case 14: CALL(14); break;        \
    default: break; /* sizes outside 2^9..2^15 samples are rejected by set_parameters */ \
  }

void launch_window_fft(const StreamDev *d_streams, int nstreams, int row0, int nrows, int nrows_total,
                       const float *window, const float2 *tw_rot, int rot, int nper, int M, int kpad, void *spec,
                       int tc_slots, float tc_scale, cudaStream_t st, int waves) {
  const int logn = 30 - __builtin_clz((unsigned)rot);  // log2(rot / 2)
#define SFXC_WIN(L)                                                                                            \
  (tc_slots == kTcSlots                                                                                         \
       ? window_fft_launch<L, kTcSlots>(d_streams, nstreams, row0, nrows, nrows_total, window, tw_rot, nper, M,  \
                                        kpad, spec, tc_scale, st, waves)                                      \
   : tc_slots == kTcSlotsWide                                                                                    \
       ? window_fft_launch<L, kTcSlotsWide>(d_streams, nstreams, row0, nrows, nrows_total, window, tw_rot, nper, \
                                            M, kpad, spec, tc_scale, st, waves)                               \
       : window_fft_launch<L, 0>(d_streams, nstreams, row0, nrows, nrows_total, window, tw_rot, nper, M, kpad,    \
                                 spec, tc_scale, st, waves))
  SFXC_LOGN_SWITCH(logn, SFXC_WIN)
#undef SFXC_WIN
}

void launch_bitstat(const StreamDev *d_streams, const int4 *d_items, int nitems, cudaStream_t st) {
  if (nitems > 0) bitstat_kernel<<<nitems, 256, 0, st>>>(d_streams, d_items, nitems);
}

void launch_phased(const float2 *spec, int nrows_total, int kpad, int nstreams, int r0, int nrows, int K, int nsub,
                   float2 *acc, cudaStream_t st) {
  phased_kernel<<<(K + 127) / 128, 128, 0, st>>>(spec, nrows_total, kpad, nstreams, r0, nrows, K, nsub, acc);
}

void launch_pc_dump(float2 *acc, float2 *pcacc, const UvShift *uvp, int nstreams, int nbl, int kpad, int K, int npc,
                    cudaStream_t st) {
  if (nbl > 0) pc_dump_kernel<<<dim3((K + 255) / 256, nbl), 256, 0, st>>>(acc, pcacc, uvp, nstreams, nbl, kpad, K, npc);
}

cudaError_t launch_reduce(const float2 *in, int nspec, int M, int nch, const float *mask, const float *lag_window,
                          int normalize, const float2 *tw2M, float2 *out, cudaStream_t st) {
  if (nspec <= 0) return cudaSuccess;
  const int logM = 31 - __builtin_clz((unsigned)M), lognch = 31 - __builtin_clz((unsigned)nch);
  const size_t smem = (size_t)M * sizeof(float2) + (size_t)2 * nch * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(reduce_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  reduce_kernel<<<nspec, 256, smem, st>>>(in, M, logM, nch, lognch, mask, lag_window, normalize, tw2M, out);
  return cudaGetLastError();
}

// Work split of the FP32 X-step for ntiles stream-pair tiles: parts of at
// most 36 tiles (12 warps x 3), the smallest tiles-per-warp that fits a part
// into 12 warps, rows per step so that a step stages at most 32 KB.
F32Plan xcorr_f32_plan(int ntiles, int npad) {
  F32Plan p;
  if (ntiles <= 0 || npad <= 0 || npad * 256 > kF32StageBytes * 4) return p;
  p.nparts = (ntiles + 35) / 36;
  p.tiles_per_part = (ntiles + p.nparts - 1) / p.nparts;
  for (p.tpw = 1; p.tpw < 3 && (p.tiles_per_part + p.tpw - 1) / p.tpw > 12; p.tpw++) {
  }
  p.warps = (p.tiles_per_part + p.tpw - 1) / p.tpw;
  p.R = std::max(1, kF32StageBytes / (npad * 256));
  p.smem = (size_t)kF32Stages * p.R * npad * 256;
  return p;
}

template <int TPW>
static void f32_launch(const F32Args &a, const F32Plan &p, bool binned, cudaStream_t st) {
  auto kern = binned ? xcorr_f32_kernel<TPW, true> : xcorr_f32_kernel<TPW, false>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
  const int nct = (a.K + 31) / 32, nrows = a.r1 - a.r0;
  const int nrb = (nrows + a.rblock - 1) / a.rblock;
  const int nitems = nct * nrb * a.nparts;
  kern<<<std::min(nitems, sm_count()), p.warps * 32, p.smem, st>>>(a);
}

// Row blocks of the unbinned FP32 X-step: about four work items per SM keep
// the CTAs balanced; each block's partial sums go to scratch and are added in
// block order.  Binned (pulsar) launches keep all rows in one block.
static int f32_row_blocks(const F32Plan &p, int K, int nrows) {
  const int nct = (K + 31) / 32;
  return std::max(1, std::min((nrows + p.R - 1) / p.R, (4 * sm_count() + nct * p.nparts - 1) / (nct * p.nparts)));
}

size_t xcorr_f32_scratch_bytes(int ntiles, int npad, int K, int nrows, int nbl, int kpad) {
  const F32Plan p = xcorr_f32_plan(ntiles, npad);
  if (p.tpw <= 0 || nrows <= 0) return 0;
  const int nrb = f32_row_blocks(p, K, nrows);
  return nrb > 1 ? (size_t)nrb * nbl * kpad * sizeof(float2) : 0;
}

void launch_xcorr_f32(const float2 *spec, int nrows_total, int kpad, int nstreams, int npad, int r0, int r1, int K,
                      const int *tiles, int ntiles, const int *blmap, int nbl, const int16_t *bins, int bins_rows,
                      float2 *acc, float2 *scratch, size_t scratch_bytes, cudaStream_t st) {
  if (r1 <= r0 || K <= 0) return;
  F32Plan p = xcorr_f32_plan(ntiles, npad);
  if (p.tpw <= 0) return;
  const bool binned = bins != nullptr;
  if (binned) {
    // binned launches keep every row of a channel in one work item (each
    // accumulator entry has one writer); finer parts of the tile set give the
    // SMs enough items (each part stages the rows again, mostly from L2)
    const int nct = (K + 31) / 32;
    const int np = std::min(ntiles, std::max(p.nparts, (2 * sm_count() + nct - 1) / nct));
    if (np > p.nparts) {
      p.nparts = np;
      p.tiles_per_part = (ntiles + np - 1) / np;
      for (p.tpw = 1; p.tpw < 3 && (p.tiles_per_part + p.tpw - 1) / p.tpw > 12; p.tpw++) {
      }
      p.warps = (p.tiles_per_part + p.tpw - 1) / p.tpw;
    }
  }
  F32Args a;
  a.spec = spec;
  a.nrows_total = nrows_total;
  a.kpad = kpad;
  a.nstreams = nstreams;
  a.npad = npad;
  a.r0 = r0;
  a.r1 = r1;
  a.K = K;
  a.tiles = tiles;
  a.ntiles = ntiles;
  a.tiles_per_part = p.tiles_per_part;
  a.nparts = p.nparts;
  a.R = p.R;
  a.blmap = blmap;
  a.nbl = nbl;
  a.bins = bins;
  a.bins_rows = bins_rows;
  a.acc = acc;
  a.part = nullptr;
  const int nrows = r1 - r0;
  int nrb = binned ? 1 : f32_row_blocks(p, K, nrows);
  if (nrb > 1 && (!scratch || scratch_bytes < (size_t)nrb * nbl * kpad * sizeof(float2))) nrb = 1;
  a.rblock = ((nrows + nrb - 1) / nrb + p.R - 1) / p.R * p.R;
  nrb = (nrows + a.rblock - 1) / a.rblock;
  if (nrb > 1) a.part = scratch;
  switch (p.tpw) {
    case 1: f32_launch<1>(a, p, binned, st); break;
    case 2: f32_launch<2>(a, p, binned, st); break;
    default: f32_launch<3>(a, p, binned, st); break;
  }
  if (nrb > 1)
    f32_part_reduce_kernel<<<dim3((K + 255) / 256, nbl), 256, 0, st>>>(scratch, nrb, nbl, kpad, K, acc);
}

void launch_pulsar_bins(int nrows, int K, double start_phase, double rate_term, double fft_duration,
                        const double *offsets, double g0, double g1, int nbins, int16_t *bins, cudaStream_t st) {
  pulsar_bins_kernel<<<dim3((nrows + 127) / 128, K), 128, 0, st>>>(nrows, K, start_phase, rate_term, fft_duration,
                                                                  offsets, g0, g1, nbins, bins);
}

void launch_normalize(const float2 *acc, int kpad, int M, int nstreams, int nbl, const int *bl, double *norms,
                      const double *flagfac, float2 *out, cudaStream_t st) {
  norm_autos_kernel<<<nstreams, 256, 0, st>>>(acc, kpad, M, nstreams, norms);
  normalize_kernel<<<dim3((M + 1 + 255) / 256, nbl), 256, 0, st>>>(acc, kpad, M, nstreams, nbl, bl, norms, flagfac,
                                                                    out);
}

}  // namespace sfxc
