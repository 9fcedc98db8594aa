// Device-side structures and helpers shared by the correlator-node kernels.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace sfxc {

constexpr int kNd = 256;  // fft_size_delaycor handled by the fused block kernel
constexpr int kTcSlots = 32;  // stream slots per (row, channel) of the tensor-core spectra layout, up to 32 streams
constexpr int kTcSlotsWide = 64;  // the same for jobs of 33 to 64 streams

// Tensor-core spectra layout, in 8-byte units (one FP16 hi/lo complex value):
// per row kpad channels x S slots (S = 32, or 64 for jobs of more than 32
// streams); the channels in groups of four, and per group the S/4 slot quads
// (slots 4q .. 4q+3) one 128-byte line each, holding the group's four
// channels x four slots.  So the four streams of a slot quad write whole
// lines, and one channel's S slots are S/4 32-byte pieces 128 bytes apart.
// kpad is a multiple of 4.
__host__ __device__ __forceinline__ int64_t tc_index(int64_t row, int kpad, int ch, int slot, int S = kTcSlots) {
  return (row * kpad + (ch & ~3)) * S + (slot >> 2) * 16 + (ch & 3) * 4 + (slot & 3);
}

// One plan segment: output samples [out0, out0+n) come from source bit src_bit
// onward (bits per sample apart); src_bit < 0 means zeros (invalid or an
// inserted sample).  Same layout as host.hpp's Segment.
struct DevSegment {
  int32_t out0, n;
  int64_t src_bit;
};
struct DevStatRange {
  int64_t src_byte;
  int32_t n, cidx;
};

// Per-block record of the F-step, written by block_params_kernel for the
// blocks of one launch.
struct BlockPar {
  // phase-ramp start (rad, [0,2pi)), ramp step per bin, fringe phase at the
  // block start, fringe phase step per sample
  float4 ph;
  // cos and sin of 16 ramp steps, cos and sin of 16 fringe steps (the
  // per-thread recurrences of the block stage)
  float4 steps;
  // bit of the block's first sample in the source when this block and the
  // next both lie inside one segment of recorded samples, else -1
  long long src_bit;
  float amp;  // amplitude at the block centre
  int32_t pad;
};
static_assert(sizeof(BlockPar) == 48, "BlockPar layout");

// Per-stream parameters of the F-step kernels (one integration).
struct StreamDev {
  const uint8_t *src;          // source bytes (protocol buffer or channel stream)
  const DevSegment *segs;      // unpack plan
  int32_t nsegs;
  int32_t bits;
  const DevStatRange *stats;   // counted-byte ranges
  int32_t nstats;
  int32_t tsys_t0, tsys_period, tsys_on0, tsys_two_bit;
  // delay model: spline over n nodes: x | (y b c d) x3 columns, 13n doubles;
  // spline_lo: the node interval of the launch's first block start, from
  // which the block kernel walks forward (no search per block)
  const double *spline;
  int32_t spline_n, spline_lo;
  int64_t scan_begin, clock_epoch;
  double clock_offset, clock_rate;
  // time base
  int64_t start_ticks;         // integration start
  int32_t tps;                 // ticks per sample
  int32_t n_blocks;            // blocks handled by this launch, starting at block0
  int32_t block0;              // first block (index within the integration)
  int64_t fft_len_ticks, half_len_ticks;
  double fft_len_sec;
  // channel setup (Delay_correction::set_parameters)
  int32_t sample_rate, bandwidth, oversamp, sideband;  // sideband +1 / -1
  double center_freq, lo_offset, start_phase;
  // per-stream quotients of Delay_correction::fractional_bit_shift, divided
  // once here: -2 pi / sample_rate and pi / (2 oversamp); the ramp terms
  // built from them end in FP32 and are computed there: -2 pi / sample_rate,
  // pi / (2 oversamp), bandwidth / 2 and sample_rate / 256 as floats
  double frac_scale, int_phase_q;
  float frac_scale_f, int_phase_q_f, half_bw_f, rate_per_bin_f;
  // -sideband * 2 pi (the fringe phase's turn-to-radian factor)
  double fringe_mult;
  // windowed FFT stage; slot: the stream's index in the job (its place in
  // the spectra layouts), also when the launch covers a subset of streams
  int32_t rot, flip, output_offset, temp_fft_offset, slot;
  // delay-model shortcuts, exact: an all-zero phase column evaluates to 0.0,
  // an all-one amplitude column to 1.0, a zero clock model to a zero drift
  int32_t phase_zero, amp_one, no_clock;
  // per-block records of this launch's blocks (block_params_kernel)
  BlockPar *bpar;
  // outputs
  float *ts;                   // fringe-stopped series, n_blocks*256 floats
  unsigned long long *hist;    // 8 code counters: cal diode on [0..3], off [4..7]
};

// --------------------------------------------------------------------------
// FP64 Akima evaluation with the same operation order as the host (no FMA
// contraction) so that integer delays agree bit for bit.
__device__ __forceinline__ int spline_index(const double *x, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int i = (hi + lo) >> 1;
    if (x[i] > v)
      hi = i;
    else
      lo = i;
  }
  return lo;
}
// The interval spline_index finds for v, walking forward from lo, an
// interval at or before it (spline_index is non-decreasing in v).
__device__ __forceinline__ int spline_walk(const double *x, int n, double v, int lo) {
  while (lo < n - 2 && x[lo + 1] <= v) lo++;
  return lo;
}
// Evaluation in node interval i (as found by spline_index or spline_walk).
__device__ __forceinline__ double spline_eval_at(const double *sp, int n, int col, double v, int i) {
  const double *x = sp;
  const double *y = sp + n + col * 4 * n;
  const double *b = y + n, *c = y + 2 * n, *d = y + 3 * n;
  double dx = __dsub_rn(v, x[i]);
  double t = __dadd_rn(c[i], __dmul_rn(d[i], dx));
  t = __dadd_rn(b[i], __dmul_rn(dx, t));
  return __dadd_rn(y[i], __dmul_rn(dx, t));
}
__device__ __forceinline__ double spline_eval(const double *sp, int n, int col, double v) {
  const double *x = sp;
  const double *y = sp + n + col * 4 * n;
  const double *b = y + n, *c = y + 2 * n, *d = y + 3 * n;
  int i = spline_index(x, n, v);
  double dx = __dsub_rn(v, x[i]);
  double t = __dadd_rn(c[i], __dmul_rn(d[i], dx));
  t = __dadd_rn(b[i], __dmul_rn(dx, t));
  return __dadd_rn(y[i], __dmul_rn(dx, t));
}
__device__ __forceinline__ double time_diff_dev(int64_t a, int64_t b) {
  return __ddiv_rn((double)(a - b), 512000000.0);
}
__device__ __forceinline__ double stream_delay(const StreamDev &s, int64_t t) {
  double r = spline_eval(s.spline, s.spline_n, 0, time_diff_dev(t, s.scan_begin));
  if (s.no_clock) return __dadd_rn(r, 0.0);
  double drift = __dadd_rn(s.clock_offset, __dmul_rn(time_diff_dev(t, s.clock_epoch), s.clock_rate));
  return __dadd_rn(r, drift);
}
__device__ __forceinline__ double stream_phase(const StreamDev &s, int64_t t) {
  return spline_eval(s.spline, s.spline_n, 1, time_diff_dev(t, s.scan_begin));
}
__device__ __forceinline__ double stream_amplitude(const StreamDev &s, int64_t t) {
  return spline_eval(s.spline, s.spline_n, 2, time_diff_dev(t, s.scan_begin));
}

// Barriers for the register FFT (fft_reg.cuh): a warp or the whole CTA.
struct WarpSync {
  __device__ void operator()() const { __syncwarp(); }
};
struct BlockSync {
  __device__ void operator()() const { __syncthreads(); }
};
// Named barrier `id` (1..15) over `count` threads (a multiple of 32) of the CTA.
struct GroupSync {
  int id, count;
  __device__ void operator()() const { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
};

// 2-bit code -> sample value, the Bit2float_worker table (sfxc/src/bit2float_worker.cc:4-10):
// 0 -> -7, 1 -> -2, 2 -> +2, 3 -> +7.  The four values differ only in their
// two high bytes (0xC0E0, 0xC000, 0x4000, 0x40E0), so one byte permute picks
// them from two table words: result byte 3 = {C0,C0,40,40}[c], byte 2 =
// {E0,00,00,E0}[c], bytes 0-1 a zero byte of the second word.
__device__ __forceinline__ float code_value2(uint32_t c) {
  return __int_as_float((int)__byte_perm(0x4040C0C0u, 0xE00000E0u, c * 0x1100u + 0x0455u));
}

// Unpacked sample `o` (index within the integration) through the plan;
// `si` is a segment cursor that only moves forward for increasing `o`.
__device__ __forceinline__ float gather_sample(const StreamDev &s, int o, int &si) {
  while (si + 1 < s.nsegs && s.segs[si].out0 + s.segs[si].n <= o) si++;
  const DevSegment sg = s.segs[si];
  if (sg.src_bit < 0 || o < sg.out0 || o >= sg.out0 + sg.n) return 0.0f;
  const int64_t bit = sg.src_bit + (int64_t)(o - sg.out0) * s.bits;
  const int code = (__ldg(s.src + (bit >> 3)) >> (bit & 7)) & ((1 << s.bits) - 1);
  // Bit2float_worker lookup tables (sfxc/src/bit2float_worker.cc:4-10)
  return s.bits == 2 ? (code == 0 ? -7.f : code == 1 ? -2.f : code == 2 ? 2.f : 7.f) : (code ? 5.f : -5.f);
}
// First segment whose range can contain sample o (binary search on out0).
__device__ __forceinline__ int find_segment(const StreamDev &s, int o) {
  int lo = 0, hi = s.nsegs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (s.segs[mid].out0 <= o)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// uvshift of one extra phase centre and cross baseline in one sub-integration:
// phase at channel 0, phase step per channel (rad), amplitude.
struct UvShift {
  double phi, delta, amp, pad;
};

// Accumulator element written by the X kernels and read by normalisation.
struct VisLayout {
  int32_t nbl, kpad;  // baselines, padded channel count
};

// One output byte of channel extraction: spb = 8 / fan_out samples from the
// spb consecutive N-byte words at w, first sample in the lowest bits; the
// subband's fan_out tracks are tr[0..fan_out) (bit positions in a word).
// Bit placement follows Channel_extractor_5 (sfxc/src/channel_extractor_5.cc:40-58,
// 67-99): track t of a sample lands at low_bit << ((t+1) % bits) with low_bit
// starting at 1 << (8 - fan_out) and advancing by `bits` per complete sample,
// and each earlier sample is shifted down by fan_out per later sample.
__device__ __forceinline__ uint8_t extract_byte(const uint8_t *w, int N, int bits, int fan_out,
                                                const int *__restrict__ tr) {
  const int spb = 8 / fan_out;
  unsigned byte = 0;
  for (int j = 0; j < spb; j++, w += N) {
    unsigned v = 0, low_bit = 1u << (8 - fan_out);
    for (int t = 0; t < fan_out; t++) {
      const int k = tr[t];
      if ((w[k >> 3] >> (k & 7)) & 1) v |= low_bit << ((t + 1) % bits);
      if ((t + 1) % bits == 0) low_bit <<= bits;
    }
    byte |= (v >> ((spb - 1 - j) * fan_out)) & 0xffu;
  }
  return (uint8_t)byte;
}

}  // namespace sfxc
