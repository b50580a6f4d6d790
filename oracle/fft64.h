/*
 * fft64.h -- double-precision DFT used by the CPU oracle (test infrastructure).
 *
 * This is NOT part of the product. It is the FP64 transform behind two
 * checkers:
 *   - oracle/tpal_oracle.c, the C restatement of the reference's
 *     Transform-PAL path, and
 *   - oracle/fftw_shim/, which exposes the subset of the FFTW3 API that the
 *     reference's transform_pal_{2d,3d}.cpp call, so those reference sources
 *     can be compiled and run here unmodified.
 *
 * The reference links FFTW 3.3.11 (pinned in its release workflow; CI uses the
 * distribution's 3.3.10). FFTW is not installed in this image, so the
 * published FFTW semantics are restated here:
 *   - forward r2c: unnormalised DFT with exponent sign -1, row-major input of
 *     n0 x n1 x ... x n_{d-1} reals, output n0 x ... x (n_{d-1}/2 + 1) complex;
 *   - backward c2r: unnormalised DFT with exponent sign +1 over the implied
 *     Hermitian-symmetric full spectrum, real output (so a round trip scales
 *     by the product of the dimensions).
 * Every transform length used on this path is a power of two (8, 16, 32).
 */
#ifndef TPO_FFT64_H
#define TPO_FFT64_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A multi-dimensional real<->complex transform plan (rank 1..3). */
typedef struct fft64_plan fft64_plan;

/* rank = number of dims; dims = sizes, row-major, each a power of two.
 * Returns NULL on an unsupported size. */
fft64_plan *fft64_plan_create(int rank, const int *dims);
void        fft64_plan_destroy(fft64_plan *p);

/* in: prod(dims) reals; out: prod(dims[0..rank-2]) * (dims[rank-1]/2+1)
 * interleaved complex (re, im). */
void fft64_r2c(const fft64_plan *p, const double *in, double *out);

/* in: half spectrum as above (not modified); out: prod(dims) reals,
 * unnormalised. */
void fft64_c2r(const fft64_plan *p, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
