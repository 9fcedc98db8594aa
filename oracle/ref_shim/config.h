/* Build configuration for compiling the reference's correlator-node classes
 * as a CPU checker (test infrastructure only; never linked into the product).
 *
 * The reference's autoconf step would generate this file; the values below
 * select its FFTW/single-precision code path (sfxc/configure.ac:45-158) with
 * sincos() available, as on any glibc system.
 */
#ifndef SFXC_REF_SHIM_CONFIG_H
#define SFXC_REF_SHIM_CONFIG_H
#define HAVE_SINCOS 1
#define PACKAGE "sfxc"
#define VERSION "ref-checker"
#endif
