/*
 * cfft.h -- CPU complex FFT used by the oracle (test infrastructure only).
 *
 * This is a plain C, double-precision, mixed-radix Stockham FFT for any
 * length n >= 1 (radix 4/2/3/5 butterflies, a direct O(p^2) DFT for any
 * other prime factor p).  It follows cuFFT's conventions as used by the
 * reference (AProductCore.cpp:47, :212-229, :719-739): forward transform
 * has sign -1, inverse has sign +1, neither is normalised, and a 3-D
 * transform of an (n0, n1, n2) array is stored with the last index fastest.
 *
 * It is the checker's FFT, never the product's: the product path runs the
 * CUDA kernels in topo-dda-forwin64_gb300/csrc.
 */
#ifndef ORACLE_CFFT_H_
#define ORACLE_CFFT_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } oc_cplx;

typedef struct oc_plan1d oc_plan1d;

/* One-dimensional plan of length n.  Returns NULL on allocation failure. */
oc_plan1d* oc_plan1d_create(int n);
void oc_plan1d_destroy(oc_plan1d* p);
int oc_plan1d_len(const oc_plan1d* p);

/* In-place transform of one line of n elements with element stride `stride`
 * (in units of oc_cplx).  sign = -1 forward, +1 inverse.  `work` must hold
 * 2*n elements. */
void oc_fft1d(const oc_plan1d* p, oc_cplx* data, ptrdiff_t stride, int sign, oc_cplx* work);

/* In-place 3-D transform of an (n0, n1, n2) array, n2 fastest, axis 2 first,
 * then axis 1, then axis 0.  Returns 0 on success. */
int oc_fft3d(int n0, int n1, int n2, oc_cplx* data, int sign);

/* The same 3-D transform, with Bluestein's chirp-z algorithm for a line
 * length that has a prime factor above 7 (the reference's 2N - 1 grids).
 * Used to time the reference's CPU path; the checker keeps oc_fft3d. */
int oc_fft3d_fast(int n0, int n1, int n2, oc_cplx* data, int sign);

#ifdef __cplusplus
}
#endif

#endif
