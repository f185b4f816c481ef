/*
 * fftw3.h — project-written stand-in for the subset of the FFTW3 double-precision
 * API that SCFT.c uses. TEST INFRASTRUCTURE ONLY: it exists so that the reference
 * solver (SCFT.c) and the CPU oracle can be compiled in an image that has no FFTW3.
 * Nothing in the GPU product includes or links it.
 *
 * Covered API (call sites in the reference): fftw_plan_dft_3d (SCFT.c:685-686,
 * :697-698), fftw_execute_dft (SCFT.c:2493, :2510, :2595, :2612), fftw_malloc /
 * fftw_free (SCFT.c:682-683, :2321-2333), fftw_destroy_plan (SCFT.c:1667-1668).
 *
 * Semantics follow FFTW's documented conventions: row-major arrays (last index
 * fastest), unnormalised transforms, FFTW_FORWARD = -1 is exp(-2*pi*i*jk/n),
 * FFTW_BACKWARD = +1. Planner flags are accepted and ignored (the arrays are
 * never touched at planning time). The algorithm is a mixed-radix decimation-
 * in-time Cooley-Tukey FFT with radix 2/3/4/5 and generic small-prime
 * butterflies, and Bluestein's chirp-z convolution for lengths with a prime
 * factor above 13 (e.g. 194 = 2*97 and 258 = 2*3*43 in Dirichlet-z runs).
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SCFT.c includes <complex.h> first, so with real FFTW fftw_complex is the C99
 * double _Complex type; the shim always uses that type. */
typedef double _Complex fftw_complex;
typedef struct offt_plan3d *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
