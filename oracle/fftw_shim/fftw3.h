/*
 * fftw3.h -- FFTW3 API shim for compiling the reference's Transform-PAL
 * sources as a CPU checker (test infrastructure, never shipped).
 *
 * Declares only the FFTW3 names that the reference's
 * src/decoders/palcolour/transform_pal_2d.cpp:176-194 and
 * src/decoders/palcolour/transform_pal_3d.cpp:195-213 (plus
 * src/common/fftw_planner.h:27-31) use. The implementation behind them is
 * oracle/fft64.c, an FP64 restatement of FFTW's published r2c/c2r semantics
 * (FFTW 3.3.11 is the version the reference pins; it is absent here).
 */
#ifndef TPO_FFTW3_SHIM_H
#define TPO_FFTW3_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct tpo_fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

double *fftw_alloc_real(unsigned long n);
fftw_complex *fftw_alloc_complex(unsigned long n);
void fftw_free(void *p);

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags);

void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
