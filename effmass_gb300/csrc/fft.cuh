// fft.cuh — block-cooperative mixed-radix Stockham FFTs on lines held in
// shared memory.
//
// The 3-D transforms of the local-potential term (the reference's FFT3D,
// src/math/fft.cppm:60-85: lines along z, then y, then x) are built from
// these.  A line of length n is transformed by a sequence of radix-p stages
// (p in {2,3,4,5,7} and any other prime up to HPSI_FFT_MAXR); stage s reads
// buffer s%2 and writes buffer (s+1)%2 (Stockham auto-sort: natural order in,
// natural order out, no bit reversal).  For a stage of radix p after stages
// whose radices multiply to Ns, butterfly i of a line reads elements
// i + q*(n/p), multiplies by W_{Ns*p}^{q*(i mod Ns)}, does a p-point DFT and
// writes to (i/Ns)*Ns*p + (i mod Ns) + q*Ns.
//
// Twiddles come from a per-length table tw[j] = exp(+2*pi*i*j/n) held in
// shared memory; the forward (R2G) sign uses its conjugate.
#pragma once

#include "common.cuh"

#define HPSI_FFT_MAXST 16
#define HPSI_FFT_MAXR 13
#define HPSI_FFT_MAXN 512

struct FftLen {
    int n;
    int nst;
    int rad[HPSI_FFT_MAXST];
};

// Factor n into stage radices, preferring 4 over 2*2.  Returns false if n has
// a prime factor above HPSI_FFT_MAXR or n exceeds HPSI_FFT_MAXN.
static inline bool fft_factor(int n, FftLen* L)
{
    L->n = n;
    L->nst = 0;
    if (n < 1 || n > HPSI_FFT_MAXN) return false;
    int m = n;
    while (m % 4 == 0) { L->rad[L->nst++] = 4; m /= 4; }
    for (int p = 2; p <= HPSI_FFT_MAXR && m > 1; ++p) {
        while (m % p == 0) {
            if (L->nst >= HPSI_FFT_MAXST) return false;
            L->rad[L->nst++] = p;
            m /= p;
        }
    }
    return m == 1;
}

// twiddle W_n^j for the given sign, from the +sign table
template <typename C>
HPSI_D C tw_get(const C* tw, int j, int sign)
{
    C w = tw[j];
    if (sign < 0) w.y = -w.y;
    return w;
}

// p-point DFT of v[0..p) in registers: v[q] <- sum_r v[r] W_p^{r q}
template <typename C, int P>
HPSI_D void dft_small(C (&v)[HPSI_FFT_MAXR], const C* tw, int n, int sign)
{
    using R = typename Real<C>::type;
    if constexpr (P == 2) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (P == 4) {
        C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        C b0 = cadd(v[1], v[3]), b1 = cmul_i(csub(v[1], v[3]), sign);
        v[0] = cadd(a0, b0);
        v[2] = csub(a0, b0);
        v[1] = cadd(a1, b1);
        v[3] = csub(a1, b1);
    } else {
        C out[P];
        const int step = n / P;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            C s = v[0];
#pragma unroll
            for (int r = 1; r < P; ++r) {
                int j = ((r * q) % P) * step;
                s = cadd(s, cmul(v[r], tw_get(tw, j, sign)));
            }
            out[q] = s;
        }
#pragma unroll
        for (int q = 0; q < P; ++q) v[q] = out[q];
        (void)sizeof(R);
    }
}

// One Stockham stage over `nl` lines.  Element e of line L lives at
// buf[L*ls + e*es].  LINE_FAST selects which index consecutive threads walk:
// lines (use when ls == 1) or butterflies (use when es == 1), so that shared
// memory accesses of a warp are contiguous.
template <typename C, int P, bool LINE_FAST>
HPSI_D void fft_stage_p(const C* __restrict__ src, C* __restrict__ dst, int n, int Ns, int nl, int ls,
                        int es, const C* tw, int sign)
{
    const int nbf = n / P;
    const int total = nl * nbf;
    const int tstep = n / (Ns * P);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int L, i;
        if (LINE_FAST) { L = t % nl; i = t / nl; }
        else { i = t % nbf; L = t / nbf; }
        const int k = i % Ns;
        C v[HPSI_FFT_MAXR];
        const C* s = src + (size_t)L * ls;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            C x = s[(size_t)(i + q * nbf) * es];
            if (q > 0 && k > 0) x = cmul(x, tw_get(tw, (q * k * tstep) % n, sign));
            v[q] = x;
        }
        dft_small<C, P>(v, tw, n, sign);
        C* d = dst + (size_t)L * ls;
        const int base = (i / Ns) * Ns * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) d[(size_t)(base + q * Ns) * es] = v[q];
    }
}

template <typename C, bool LINE_FAST>
HPSI_D void fft_stage(const C* src, C* dst, int p, int n, int Ns, int nl, int ls, int es, const C* tw, int sign)
{
    switch (p) {
        case 2: fft_stage_p<C, 2, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 3: fft_stage_p<C, 3, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 4: fft_stage_p<C, 4, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 5: fft_stage_p<C, 5, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 7: fft_stage_p<C, 7, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 11: fft_stage_p<C, 11, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        case 13: fft_stage_p<C, 13, LINE_FAST>(src, dst, n, Ns, nl, ls, es, tw, sign); break;
        default: break;  // fft_factor admits no other radix
    }
}

// Full transform of nl lines; data starts in bufs[cur] and the function
// returns the index (0/1) of the buffer holding the result.
template <typename C, bool LINE_FAST>
HPSI_D int fft_lines(C* buf0, C* buf1, int cur, const FftLen& L, int nl, int ls, int es, const C* tw, int sign)
{
    int Ns = 1;
    for (int s = 0; s < L.nst; ++s) {
        const int p = L.rad[s];
        C* src = cur ? buf1 : buf0;
        C* dst = cur ? buf0 : buf1;
        fft_stage<C, LINE_FAST>(src, dst, p, L.n, Ns, nl, ls, es, tw, sign);
        __syncthreads();
        Ns *= p;
        cur ^= 1;
    }
    return cur;
}
