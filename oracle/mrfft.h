/*
 * mrfft.h — project-written mixed-radix complex FFT in FP64 (test infrastructure).
 *
 * This is the oracle's 1-D transform.  It is used twice:
 *   1. by oracle/hpsi_oracle.c (the CPU restatement of the H|psi> path), and
 *   2. behind the pocketfft C API that the reference calls at
 *      src/math/fft.cppm:29-41 (make_cfft_plan / cfft_forward / cfft_backward),
 *      because the reference's vendor/pocketfft submodule is empty.
 *
 * Conventions follow pocketfft's C interface: data are interleaved (re, im)
 * doubles; forward uses exp(-2*pi*i*j*k/n), backward exp(+2*pi*i*j*k/n);
 * the result is multiplied by `fct`.  The algorithm is a recursive
 * decimation-in-time Cooley-Tukey over the prime factors of n with an exact
 * twiddle table (cos/sin evaluated directly for every index, no recurrence),
 * so the rounding error grows like eps*log(n).
 */
#ifndef HPSI_ORACLE_MRFFT_H
#define HPSI_ORACLE_MRFFT_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MRFFT_MAXFAC 64
#define MRFFT_MAXP 64

typedef struct mrfft_plan_s {
    int n;
    int nfac;
    int fac[MRFFT_MAXFAC];
    double *tw;   /* [2n]: cos(2*pi*j/n), sin(2*pi*j/n); read-only after mrfft_make */
} mrfft_plan_s;

static inline mrfft_plan_s *mrfft_make(int n)
{
    if (n < 1) return NULL;
    mrfft_plan_s *p = (mrfft_plan_s *)calloc(1, sizeof(mrfft_plan_s));
    if (!p) return NULL;
    p->n = n;
    int m = n, f = 2;
    while (m > 1) {
        while (m % f != 0) ++f;
        if (f > MRFFT_MAXP || p->nfac >= MRFFT_MAXFAC) { free(p); return NULL; }
        p->fac[p->nfac++] = f;
        m /= f;
    }
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p->tw) { free(p); return NULL; }
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < n; ++j) {
        double a = two_pi * (double)j / (double)n;
        p->tw[2 * j] = cos(a);
        p->tw[2 * j + 1] = sin(a);
    }
    return p;
}

static inline void mrfft_free(mrfft_plan_s *p)
{
    if (!p) return;
    free(p->tw);
    free(p);
}

/* out[0..len) = DFT of in[0, istride, 2*istride, ...] with factors fac[fi..] */
static void mrfft_rec(const mrfft_plan_s *P, const double *in, double *out, double *work,
                      int len, int istride, int fi, int sign)
{
    if (len == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    const int p = P->fac[fi];
    const int m = len / p;
    for (int r = 0; r < p; ++r)
        mrfft_rec(P, in + 2 * (size_t)r * istride, out + 2 * (size_t)r * m, work, m, istride * p, fi + 1, sign);

    const int N = P->n;
    const int tstep = N / len;     /* W_len^j = W_N^(j*tstep) */
    const int pstep = N / p;       /* W_p^j   = W_N^(j*pstep) */
    double xr[MRFFT_MAXP], xi[MRFFT_MAXP];
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            double ar = out[2 * ((size_t)r * m + k)];
            double ai = out[2 * ((size_t)r * m + k) + 1];
            long j = ((long)r * k * tstep) % N;
            double wr = P->tw[2 * j], wi = sign * P->tw[2 * j + 1];
            xr[r] = ar * wr - ai * wi;
            xi[r] = ar * wi + ai * wr;
        }
        for (int q = 0; q < p; ++q) {
            double sr = 0.0, si = 0.0;
            for (int r = 0; r < p; ++r) {
                long j = ((long)r * q * pstep) % N;
                double wr = P->tw[2 * j], wi = sign * P->tw[2 * j + 1];
                sr += xr[r] * wr - xi[r] * wi;
                si += xr[r] * wi + xi[r] * wr;
            }
            work[2 * ((size_t)q * m + k)] = sr;
            work[2 * ((size_t)q * m + k) + 1] = si;
        }
    }
    /* children finished before this level started, so one scratch serves all levels */
    memcpy(out, work, sizeof(double) * 2 * (size_t)len);
}

/* In-place transform of n interleaved complex values; sign=-1 forward, +1 backward.
 * The plan is read-only here, so one plan may serve several threads. */
static inline void mrfft_exec(const mrfft_plan_s *P, double *c, int sign, double fct)
{
    const int n = P->n;
    if (n == 1) { c[0] *= fct; c[1] *= fct; return; }
    double *tmp = (double *)malloc(sizeof(double) * 4 * (size_t)n);
    mrfft_rec(P, c, tmp, tmp + 2 * (size_t)n, n, 1, 0, sign);
    for (int j = 0; j < 2 * n; ++j) c[j] = tmp[j] * fct;
    free(tmp);
}

#ifdef __cplusplus
}
#endif
#endif
