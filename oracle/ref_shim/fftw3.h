/* Minimal FFTW3 single-precision API for building the reference's FFT
 * wrapper (sfxc/src/sfxc_fft_float.cc:103-243) without libfftw3f.
 *
 * Test infrastructure only.  The transforms follow FFTW's documented
 * conventions: unnormalised, forward sign -1, backward sign +1, r2c writes
 * n/2+1 bins, c2r reads n/2+1 bins.  They are computed in double precision
 * (fftw_shim.cc) and rounded to float, so they are at least as accurate as
 * FFTW's own float transforms.
 */
#ifndef SFXC_REF_SHIM_FFTW3_H
#define SFXC_REF_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct sfxc_shim_plan_s *fftwf_plan;
typedef struct sfxc_shim_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif
#endif
