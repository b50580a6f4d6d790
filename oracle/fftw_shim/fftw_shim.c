/*
 * fftw_shim.c -- the FFTW3 subset declared in fftw3.h, implemented on the
 * oracle's FP64 transform (oracle/fft64.c). Test infrastructure only.
 */
#include "fftw3.h"

#include <stdlib.h>

#include "../fft64.h"

struct tpo_fftw_plan_s {
    fft64_plan *plan;
    int r2c; /* 1: real in -> complex out; 0: complex in -> real out */
    void *in;
    void *out;
};

double *fftw_alloc_real(unsigned long n) { return (double *)malloc(sizeof(double) * (n ? n : 1)); }
fftw_complex *fftw_alloc_complex(unsigned long n) { return (fftw_complex *)malloc(sizeof(fftw_complex) * (n ? n : 1)); }
void fftw_free(void *p) { free(p); }

static fftw_plan make(int rank, const int *dims, int r2c, void *in, void *out)
{
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->plan = fft64_plan_create(rank, dims);
    if (!p->plan) {
        free(p);
        return NULL;
    }
    p->r2c = r2c;
    p->in = in;
    p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    const int d[2] = {n0, n1};
    return make(2, d, 1, in, out);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    const int d[2] = {n0, n1};
    return make(2, d, 0, in, out);
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    const int d[3] = {n0, n1, n2};
    return make(3, d, 1, in, out);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    const int d[3] = {n0, n1, n2};
    return make(3, d, 0, in, out);
}

void fftw_execute(const fftw_plan p)
{
    if (p->r2c) fft64_r2c(p->plan, (const double *)p->in, (double *)p->out);
    else fft64_c2r(p->plan, (const double *)p->in, (double *)p->out);
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    fft64_plan_destroy(p->plan);
    free(p);
}
