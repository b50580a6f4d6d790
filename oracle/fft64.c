/*
 * fft64.c -- FP64 multi-dimensional real DFT for the CPU oracle.
 *
 * Test infrastructure only (see fft64.h). Radix-2 iterative complex FFT with
 * double twiddles from libm; the multi-dimensional real transforms run the
 * last axis as a complex FFT of real data (keeping bins 0..n/2) and then
 * complex FFTs along the remaining axes, which is the row-major r2c/c2r
 * contract FFTW documents for fftw_plan_dft_r2c_{2d,3d} and
 * fftw_plan_dft_c2r_{2d,3d}.
 */
#define _GNU_SOURCE
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define FFT64_MAX_RANK 3
#define FFT64_MAX_N 64

struct fft64_plan {
    int rank;
    int dims[FFT64_MAX_RANK];
    int half;              /* dims[rank-1]/2 + 1 */
    size_t nreal;          /* prod(dims) */
    size_t ncplx;          /* prod(dims[0..rank-2]) * half */
    double *work;          /* ncplx complex scratch */
    double line[2 * FFT64_MAX_N];
    /* twiddles exp(-2 pi i k / n) for each distinct axis length */
    double tw[FFT64_MAX_RANK][FFT64_MAX_N];
};

static int is_pow2(int n) { return n >= 1 && (n & (n - 1)) == 0; }

/* In-place radix-2 complex FFT of length n on interleaved data.
 * sign = -1 forward, +1 backward (unnormalised). tw holds exp(-2pi i k/n),
 * k < n/2, as (cos, sin) pairs. */
static void cfft(double *x, int n, const double *tw, int sign)
{
    /* bit reversal */
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j];
            x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr;
            x[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const int halfLen = len >> 1;
        const int step = n / len;
        for (int base = 0; base < n; base += len) {
            for (int k = 0; k < halfLen; k++) {
                const double wr = tw[2 * (k * step)];
                const double wi = (sign < 0) ? tw[2 * (k * step) + 1] : -tw[2 * (k * step) + 1];
                double *a = x + 2 * (base + k);
                double *b = x + 2 * (base + k + halfLen);
                const double br = b[0] * wr - b[1] * wi;
                const double bi = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br;
                b[1] = a[1] - bi;
                a[0] = a[0] + br;
                a[1] = a[1] + bi;
            }
        }
    }
}

fft64_plan *fft64_plan_create(int rank, const int *dims)
{
    if (rank < 1 || rank > FFT64_MAX_RANK) return NULL;
    for (int d = 0; d < rank; d++) {
        if (!is_pow2(dims[d]) || dims[d] > FFT64_MAX_N || dims[d] < 2) return NULL;
    }
    fft64_plan *p = (fft64_plan *)calloc(1, sizeof(fft64_plan));
    if (!p) return NULL;
    p->rank = rank;
    p->nreal = 1;
    for (int d = 0; d < rank; d++) {
        p->dims[d] = dims[d];
        p->nreal *= (size_t)dims[d];
        const int n = dims[d];
        /* tw stores n/2 complex pairs in n doubles */
        for (int k = 0; k < n / 2; k++) {
            const double a = -2.0 * M_PI * (double)k / (double)n;
            p->tw[d][2 * k] = cos(a);
            p->tw[d][2 * k + 1] = sin(a);
        }
    }
    p->half = dims[rank - 1] / 2 + 1;
    p->ncplx = (p->nreal / (size_t)dims[rank - 1]) * (size_t)p->half;
    p->work = (double *)malloc(sizeof(double) * 2 * p->ncplx);
    if (!p->work) {
        free(p);
        return NULL;
    }
    return p;
}

void fft64_plan_destroy(fft64_plan *p)
{
    if (!p) return;
    free(p->work);
    free(p);
}

/* Complex FFTs along axis d (d < rank-1) of a half-spectrum array. */
static void axis_pass(fft64_plan *p, double *spec, int d, int sign)
{
    const int n = p->dims[d];
    /* stride (in complex elements) of axis d in the half-spectrum layout */
    size_t stride = (size_t)p->half;
    for (int e = p->rank - 2; e > d; e--) stride *= (size_t)p->dims[e];
    size_t outer = 1;
    for (int e = 0; e < d; e++) outer *= (size_t)p->dims[e];
    double *line = p->line;
    for (size_t o = 0; o < outer; o++) {
        double *blk = spec + 2 * o * stride * (size_t)n;
        for (size_t s = 0; s < stride; s++) {
            for (int i = 0; i < n; i++) {
                line[2 * i] = blk[2 * (s + (size_t)i * stride)];
                line[2 * i + 1] = blk[2 * (s + (size_t)i * stride) + 1];
            }
            cfft(line, n, p->tw[d], sign);
            for (int i = 0; i < n; i++) {
                blk[2 * (s + (size_t)i * stride)] = line[2 * i];
                blk[2 * (s + (size_t)i * stride) + 1] = line[2 * i + 1];
            }
        }
    }
}

void fft64_r2c(const fft64_plan *cp, const double *in, double *out)
{
    fft64_plan *p = (fft64_plan *)cp;
    const int n = p->dims[p->rank - 1];
    const size_t rows = p->nreal / (size_t)n;
    double *line = p->line;
    for (size_t r = 0; r < rows; r++) {
        for (int i = 0; i < n; i++) {
            line[2 * i] = in[r * (size_t)n + (size_t)i];
            line[2 * i + 1] = 0.0;
        }
        cfft(line, n, p->tw[p->rank - 1], -1);
        memcpy(out + 2 * r * (size_t)p->half, line, sizeof(double) * 2 * (size_t)p->half);
    }
    for (int d = p->rank - 2; d >= 0; d--) axis_pass(p, out, d, -1);
}

void fft64_c2r(const fft64_plan *cp, const double *in, double *out)
{
    fft64_plan *p = (fft64_plan *)cp;
    const int n = p->dims[p->rank - 1];
    const size_t rows = p->nreal / (size_t)n;
    memcpy(p->work, in, sizeof(double) * 2 * p->ncplx);
    for (int d = 0; d <= p->rank - 2; d++) axis_pass(p, p->work, d, +1);
    double *line = p->line;
    for (size_t r = 0; r < rows; r++) {
        const double *h = p->work + 2 * r * (size_t)p->half;
        for (int k = 0; k < p->half; k++) {
            line[2 * k] = h[2 * k];
            line[2 * k + 1] = h[2 * k + 1];
        }
        for (int k = 1; k < n / 2; k++) {
            line[2 * (n - k)] = h[2 * k];
            line[2 * (n - k) + 1] = -h[2 * k + 1];
        }
        cfft(line, n, p->tw[p->rank - 1], +1);
        for (int i = 0; i < n; i++) out[r * (size_t)n + (size_t)i] = line[2 * i];
    }
}
