// Register-resident FFT building blocks for the F-step kernels.
//
// A transform of N = 2^LOGN complex points is done by T = N/16 cooperating
// threads that each hold 16 values in registers.  Passes are radix-16
// Stockham steps (and one final radix-2/4/8 step when LOGN is not a multiple
// of 4) computed in registers; between passes the values go through one
// shared buffer of N + N/16 float2.  The padded index i + i/16 keeps both
// access patterns of a pass -- unit stride across threads and stride 16
// within a thread -- free of shared-memory bank conflicts.
#pragma once
#include <cuda_runtime.h>

namespace sfxc {

__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * w (SIGN < 0) or a * conj(w) (SIGN > 0), w = exp(-2 pi i m / N) from a table
template <int SIGN>
__device__ __forceinline__ float2 cmulw(float2 a, float2 w) {
  const float wi = SIGN < 0 ? w.y : -w.y;
  return make_float2(a.x * w.x - a.y * wi, a.x * wi + a.y * w.x);
}
// d * (-i) for the forward transform, d * (+i) for the backward one
template <int SIGN>
__device__ __forceinline__ float2 rot90(float2 d) {
  return SIGN < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
}
// multiplication by exp(SIGN 2 pi i m / 16) for the constant twiddles of the 16-point kernel
template <int SIGN, int M>
__device__ __forceinline__ float2 w16(float2 a) {
  constexpr float C1 = 0.92387953251128674f, S1 = 0.38268343236508978f, R2 = 0.70710678118654752f;
  constexpr int m = M & 15;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (m == 4) {
    return rot90<SIGN>(a);
  } else if constexpr (m == 8) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (m == 12) {
    return rot90<-SIGN>(a);
  } else {
    static_assert(m == 1 || m == 2 || m == 3 || m == 6 || m == 9, "twiddle not needed");
    // cos and the sine of the forward (negative) exponent
    constexpr float c = m == 1 ? C1 : m == 2 ? R2 : m == 3 ? S1 : m == 6 ? -R2 : -C1;
    constexpr float sn = m == 1 ? -S1 : m == 2 ? -R2 : m == 3 ? -C1 : m == 6 ? -R2 : S1;
    return cmul(a, make_float2(c, SIGN < 0 ? sn : -sn));
  }
}

template <int SIGN>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
// in-place 4-point DFT of (a0, a1, a2, a3), outputs in natural order
template <int SIGN>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3) {
  const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = rot90<SIGN>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}
template <int SIGN>
__device__ __forceinline__ void dft8(float2 *v) {
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<SIGN>(e0, e1, e2, e3);
  dft4<SIGN>(o0, o1, o2, o3);
  o1 = w16<SIGN, 2>(o1);
  o2 = w16<SIGN, 4>(o2);
  o3 = w16<SIGN, 6>(o3);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}
// 16-point DFT as 4 x 4: x[n1 + 4 n2] -> X[k1 + 4 k2].  upper_zero: the
// caller guarantees v[9..15] == 0, so the first 4-point stage drops the
// additions of zeros (same results).
template <int SIGN>
__device__ __forceinline__ void dft16(float2 (&v)[16], bool upper_zero = false) {
  if (upper_zero) {
    {  // (v0, v4, v8, 0)
      const float2 t0 = cadd(v[0], v[8]), t1 = csub(v[0], v[8]), t3 = rot90<SIGN>(v[4]);
      v[8] = csub(t0, v[4]);
      v[0] = cadd(t0, v[4]);
      v[4] = cadd(t1, t3);
      v[12] = csub(t1, t3);
    }
#pragma unroll
    for (int n1 = 1; n1 < 4; n1++) {  // (v[n1], v[n1 + 4], 0, 0)
      const float2 a = v[n1], b = v[n1 + 4], rb = rot90<SIGN>(b);
      v[n1] = cadd(a, b);
      v[n1 + 8] = csub(a, b);
      v[n1 + 4] = cadd(a, rb);
      v[n1 + 12] = csub(a, rb);
    }
  } else {
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) dft4<SIGN>(v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]);
  }
  // v[n1 + 4 k1] = y[n1][k1]; twiddle W16^(n1 k1)
  v[5] = w16<SIGN, 1>(v[5]);
  v[9] = w16<SIGN, 2>(v[9]);
  v[13] = w16<SIGN, 3>(v[13]);
  v[6] = w16<SIGN, 2>(v[6]);
  v[10] = w16<SIGN, 4>(v[10]);
  v[14] = w16<SIGN, 6>(v[14]);
  v[7] = w16<SIGN, 3>(v[7]);
  v[11] = w16<SIGN, 6>(v[11]);
  v[15] = w16<SIGN, 9>(v[15]);
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) dft4<SIGN>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  // v[4 k1 + k2] = X[k1 + 4 k2]: transpose into natural order
  float2 o[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) o[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = o[i];
}

// v[r] *= W^(r m) for r = 1..15 given w1, w2, w4, w8 = W^m, W^2m, W^4m, W^8m
// (W = exp(-2 pi i / N), conjugated for SIGN > 0); at most three products
// per twiddle.
template <int SIGN>
__device__ __forceinline__ void twiddle16(float2 (&v)[16], float2 w1, float2 w2, float2 w4, float2 w8) {
  const float2 w3 = cmul(w1, w2), w5 = cmul(w4, w1), w6 = cmul(w4, w2), w7 = cmul(w4, w3);
  const float2 w[8] = {make_float2(1.f, 0.f), w1, w2, w3, w4, w5, w6, w7};
#pragma unroll
  for (int r = 1; r < 8; r++) v[r] = cmulw<SIGN>(v[r], w[r]);
  v[8] = cmulw<SIGN>(v[8], w8);
#pragma unroll
  for (int r = 9; r < 16; r++) v[r] = cmulw<SIGN>(v[r], cmul(w8, w[r - 8]));
}

// Twiddles of the radix-16 passes after the first, in shared memory.  The
// pass of stride Ns (16, 256, ...) uses entries e = (Ns - 16) / 15 + k for
// k < Ns, L = pass_table_len<LOGN>() entries in all; m = k N / (16 Ns) and
// W = exp(-2 pi i / N).  Three layouts (TWK):
//   15: tab[(r - 1) L + e] = W^(r m), r = 1..15, 15 L float2: every twiddle
//       a correctly rounded table value, no products;
//    8: tab[j L + e] = {W^(2j+1)m, W^(2j+2)m}, j < 4, 4 L float4: the first
//       eight, the other seven as products with W^8m;
//    4: tab[e] = {W^m, W^2m}, tab[L + e] = {W^4m, W^8m}, 2 L float4: a quarter
//       of the space, the other eleven twiddles as products of these.
// Either way consecutive threads read consecutive entries (no bank conflicts).
template <int LOGN>
__host__ __device__ constexpr int pass_table_len() {
  int n = 1;
  for (int p = 0; p < LOGN / 4; p++) n *= 16;
  return (n - 16) / 15;
}
template <int LOGN, int TWK>
__host__ __device__ constexpr int pass_table_bytes() {
  return pass_table_len<LOGN>() * (TWK == 15 ? 15 * 8 : TWK == 8 ? 64 : 32);
}
// Fill the table from tw[j] = exp(-2 pi i j / N) by threads tid = 0..nthr-1
// (the caller synchronises before use).
template <int LOGN, int TWK>
__device__ __forceinline__ void fill_pass_table(void *tab, const float2 *__restrict__ tw, int tid, int nthr) {
  constexpr int N = 1 << LOGN, L = pass_table_len<LOGN>();
  static_assert(TWK == 4 || TWK == 8 || TWK == 15, "table layout");
  auto m_of = [](int e) {
    int Ns = 16;
    while (e >= (16 * Ns - 16) / 15) Ns *= 16;
    return (e - (Ns - 16) / 15) * (N / (16 * Ns));
  };
  if constexpr (TWK == 15) {
    float2 *t15 = static_cast<float2 *>(tab);
    for (int i = tid; i < 15 * L; i += nthr) t15[i] = __ldg(tw + (1 + i / L) * m_of(i % L));  // r m < N
  } else if constexpr (TWK == 8) {
    float4 *t8 = static_cast<float4 *>(tab);
    for (int i = tid; i < 4 * L; i += nthr) {
      const int j = i / L, m = m_of(i % L);
      const float2 a = __ldg(tw + (2 * j + 1) * m), b = __ldg(tw + (2 * j + 2) * m);  // 8 m < N
      t8[i] = make_float4(a.x, a.y, b.x, b.y);
    }
  } else {
    float4 *t4 = static_cast<float4 *>(tab);
    for (int e = tid; e < L; e += nthr) {
      const int m = m_of(e);
      const float2 w1 = __ldg(tw + m), w2 = __ldg(tw + 2 * m), w4 = __ldg(tw + 4 * m), w8 = __ldg(tw + 8 * m);
      t4[e] = make_float4(w1.x, w1.y, w2.x, w2.y);
      t4[L + e] = make_float4(w4.x, w4.y, w8.x, w8.y);
    }
  }
}

// Transform of N = 2^LOGN points by T = N/16 threads (t = 0..T-1).
// In: v[r] = x[t + r T].  `sm`: this transform's buffer of padi(N) float2.
// `tw`: exp(-2 pi i j / N) for j < N (final radix-2/4/8 pass); `ptab`: the
// radix-16 passes' table of layout TWK in shared memory (fill_pass_table).  `sync` is the
// barrier over all threads sharing the barrier (warp or CTA); every one of
// them must call this.
// Out (TO_SMEM): X[k] at sm[padi(k)], visible after the final barrier.
// Out (!TO_SMEM, LOGN % 4 == 0 only): v[r] = X[t + r T]; sm is free again
// once every thread has returned (the caller syncs before reusing it).
// upper_zero: v[9..15] == 0 on entry (the first pass skips those additions).
template <int SIGN, int LOGN, bool TO_SMEM, int TWK, typename Sync>
__device__ __forceinline__ void fft_reg(float2 (&v)[16], float2 *sm, int t, const float2 *__restrict__ tw,
                                        const void *ptab, Sync sync, bool upper_zero = false) {
  constexpr int N = 1 << LOGN, T = N / 16, NR16 = LOGN / 4, LAST = LOGN % 4;
  static_assert(NR16 >= 1, "at least 16 points");
  static_assert(TO_SMEM || LAST == 0, "register output needs a final radix-16 pass");
  // T, Q and every stride Ns >= 16 are multiples of 16, and the Ns = 1 pass
  // writes 16 consecutive entries from a multiple of 16, so each padded index
  // is padi(base) plus a compile-time offset (padi(x + 16 m) = padi(x) + 17 m)
  const int rbase = padi(t);
  int Ns = 1;
#pragma unroll
  for (int p = 0; p < NR16; p++) {
    if (p > 0) {
#pragma unroll
      for (int r = 0; r < 16; r++) v[r] = sm[rbase + r * (T + T / 16)];
      sync();
      constexpr int L = pass_table_len<LOGN>();
      const int e = (Ns - 16) / 15 + (t & (Ns - 1));
      if constexpr (TWK == 15) {
        const float2 *pt = static_cast<const float2 *>(ptab) + e;
#pragma unroll
        for (int r = 1; r < 16; r++) v[r] = cmulw<SIGN>(v[r], pt[(r - 1) * L]);
      } else if constexpr (TWK == 8) {
        const float4 *pt = static_cast<const float4 *>(ptab) + e;
        float2 w[8];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float4 q = pt[j * L];
          w[2 * j] = make_float2(q.x, q.y);
          w[2 * j + 1] = make_float2(q.z, q.w);
        }
        // w[r - 1] = W^(r m), r = 1..8
#pragma unroll
        for (int r = 1; r <= 8; r++) v[r] = cmulw<SIGN>(v[r], w[r - 1]);
#pragma unroll
        for (int r = 9; r < 16; r++) v[r] = cmulw<SIGN>(v[r], cmul(w[7], w[r - 9]));
      } else {
        const float4 a = static_cast<const float4 *>(ptab)[e], b = static_cast<const float4 *>(ptab)[L + e];
        twiddle16<SIGN>(v, make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(b.x, b.y),
                        make_float2(b.z, b.w));
      }
    }
    dft16<SIGN>(v, p == 0 && upper_zero);
    if (p == NR16 - 1 && LAST == 0 && !TO_SMEM) return;  // v[r] = X[t + r T]
    const int wbase = padi((t - (t & (Ns - 1))) * 16 + (t & (Ns - 1)));
#pragma unroll
    for (int r = 0; r < 16; r++) sm[wbase + r * (Ns + Ns / 16)] = v[r];
    sync();
    Ns *= 16;
  }
  if constexpr (LAST > 0) {
    constexpr int R = 1 << LAST, G = 16 / R, Q = N / R;  // Ns == Q here
#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int r = 0; r < R; r++) v[g * R + r] = sm[rbase + g * (T + T / 16) + r * (Q + Q / 16)];
    sync();
#pragma unroll
    for (int g = 0; g < G; g++) {
      const int j = t + g * T;
      float2 *u = v + g * R;
      if constexpr (R == 2) {
        u[1] = cmulw<SIGN>(u[1], __ldg(tw + j));
        dft2<SIGN>(u[0], u[1]);
      } else if constexpr (R == 4) {
        const float2 w1 = __ldg(tw + j), w2 = __ldg(tw + 2 * j);
        u[1] = cmulw<SIGN>(u[1], w1);
        u[2] = cmulw<SIGN>(u[2], w2);
        u[3] = cmulw<SIGN>(u[3], cmul(w1, w2));
        dft4<SIGN>(u[0], u[1], u[2], u[3]);
      } else {
        const float2 w1 = __ldg(tw + j), w2 = __ldg(tw + 2 * j), w4 = __ldg(tw + 4 * j);
        const float2 w3 = cmul(w1, w2);
        u[1] = cmulw<SIGN>(u[1], w1);
        u[2] = cmulw<SIGN>(u[2], w2);
        u[3] = cmulw<SIGN>(u[3], w3);
        u[4] = cmulw<SIGN>(u[4], w4);
        u[5] = cmulw<SIGN>(u[5], cmul(w4, w1));
        u[6] = cmulw<SIGN>(u[6], cmul(w4, w2));
        u[7] = cmulw<SIGN>(u[7], cmul(w4, w3));
        dft8<SIGN>(u);
      }
#pragma unroll
      for (int r = 0; r < R; r++) sm[rbase + g * (T + T / 16) + r * (Q + Q / 16)] = u[r];
    }
    sync();
  }
}

}  // namespace sfxc
