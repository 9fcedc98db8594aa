// FFTW3 single-precision API implemented with a double-precision FFT.
// Test infrastructure for building the reference's own FFT wrapper
// (sfxc/src/sfxc_fft_float.cc:103-243) as a CPU checker; never part of the
// product.  Conventions follow FFTW's documentation: unnormalised, forward
// sign -1, backward sign +1, r2c produces n/2+1 bins, c2r consumes n/2+1 bins
// (imaginary parts of DC and Nyquist ignored).
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstdlib>
#include <vector>

typedef std::complex<double> cd;

struct sfxc_shim_plan_s {
  int n;
  int kind;  // 0 = c2c, 1 = r2c, 2 = c2r
  int sign;
  std::vector<cd> tw;  // exp(sign * 2 pi i k / n), k < n
};

static void fft_inplace(std::vector<cd> &a, int sign, const std::vector<cd> &tw) {
  const int n = (int)a.size();
  if (n & (n - 1)) {  // not a power of two: direct DFT
    std::vector<cd> out(n);
    for (int k = 0; k < n; k++) {
      cd s = 0;
      for (int j = 0; j < n; j++) s += a[j] * tw[(long long)j * k % n];
      out[k] = s;
    }
    a.swap(out);
    return;
  }
  for (int i = 1, j = 0; i < n; i++) {  // bit reversal
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int step = n / len;
    for (int i = 0; i < n; i += len) {
      for (int j = 0; j < len / 2; j++) {
        cd u = a[i + j];
        cd v = a[i + j + len / 2] * tw[j * step];
        a[i + j] = u + v;
        a[i + j + len / 2] = u - v;
      }
    }
  }
  (void)sign;
}

static fftwf_plan make_plan(int n, int kind, int sign) {
  sfxc_shim_plan_s *p = new sfxc_shim_plan_s;
  p->n = n;
  p->kind = kind;
  p->sign = sign;
  p->tw.resize(n);
  for (int k = 0; k < n; k++) {
    double ang = sign * 2.0 * M_PI * (double)k / (double)n;
    p->tw[k] = cd(std::cos(ang), std::sin(ang));
  }
  return p;
}

extern "C" {

void *fftwf_malloc(size_t n) { return std::malloc(n ? n : 1); }
void fftwf_free(void *p) { std::free(p); }

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *, fftwf_complex *, int sign, unsigned) {
  return make_plan(n, 0, sign);
}
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *, fftwf_complex *, unsigned) {
  return make_plan(n, 1, FFTW_FORWARD);
}
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *, float *, unsigned) {
  return make_plan(n, 2, FFTW_BACKWARD);
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) {
  std::vector<cd> a(p->n);
  for (int i = 0; i < p->n; i++) a[i] = cd(in[i][0], in[i][1]);
  fft_inplace(a, p->sign, p->tw);
  for (int i = 0; i < p->n; i++) {
    out[i][0] = (float)a[i].real();
    out[i][1] = (float)a[i].imag();
  }
}

void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) {
  std::vector<cd> a(p->n);
  for (int i = 0; i < p->n; i++) a[i] = cd(in[i], 0.0);
  fft_inplace(a, p->sign, p->tw);
  for (int i = 0; i <= p->n / 2; i++) {
    out[i][0] = (float)a[i].real();
    out[i][1] = (float)a[i].imag();
  }
}

void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) {
  const int n = p->n;
  std::vector<cd> a(n);
  for (int i = 0; i <= n / 2; i++) a[i] = cd(in[i][0], in[i][1]);
  a[0] = cd(a[0].real(), 0.0);
  if (n % 2 == 0) a[n / 2] = cd(a[n / 2].real(), 0.0);
  for (int i = n / 2 + 1; i < n; i++) a[i] = std::conj(a[n - i]);
  fft_inplace(a, p->sign, p->tw);
  for (int i = 0; i < n; i++) out[i] = (float)a[i].real();
}

void fftwf_destroy_plan(fftwf_plan p) { delete p; }

}  // extern "C"
