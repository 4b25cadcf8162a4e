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

// Division by a run-time constant d (dividends below 2^31) as a multiply-high
// and a shift: q = (umulhi(x, mul) + x) >> shr (Granlund-Montgomery).
struct FastDiv {
    uint32_t d, mul, shr;
};

static inline FastDiv make_fastdiv(uint32_t d)
{
    FastDiv f{d, 0u, 0u};
    if (d <= 1) return f;
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    f.shr = l;
    f.mul = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    return f;
}

HPSI_D uint32_t fdiv(uint32_t x, const FastDiv& f) { return (__umulhi(x, f.mul) + x) >> f.shr; }

struct FftLen {
    int n;
    int nst;
    int rad[HPSI_FFT_MAXST];
    FastDiv ns[HPSI_FFT_MAXST];  // divisor by the product of the radices before stage s
};

// Factor n into stage radices, preferring the composite radices 8 and 9
// (fewest stages: 72 = 8*9), then 4, then primes.  Returns false if n has a
// prime factor above HPSI_FFT_MAXR or n exceeds HPSI_FFT_MAXN.
static inline bool fft_factor(int n, FftLen* L)
{
    L->n = n;
    L->nst = 0;
    if (n < 1 || n > HPSI_FFT_MAXN) return false;
    int m = n;
    const int pref[3] = {8, 9, 4};
    for (int r : pref)
        while (m % r == 0 && L->nst < HPSI_FFT_MAXST) { L->rad[L->nst++] = r; m /= r; }
    for (int p = 2; p <= HPSI_FFT_MAXR && m > 1; ++p) {
        while (m % p == 0) {
            if (L->nst >= HPSI_FFT_MAXST) return false;
            L->rad[L->nst++] = p;
            m /= p;
        }
    }
    int Ns = 1;
    for (int s = 0; s < L->nst; ++s) {
        L->ns[s] = make_fastdiv((uint32_t)Ns);
        Ns *= L->rad[s];
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

// 3-point DFT of (a, b, c) in place with W_3 = exp(sign*2*pi*i/3)
template <typename C>
HPSI_D void dft3(C& a, C& b, C& c, int sign)
{
    using R = typename Real<C>::type;
    const R h = (R)0.86602540378443864676;  // sin(2 pi/3)
    C s = cadd(b, c), d = csub(b, c);
    C a0 = a;
    a = cadd(a0, s);
    C m = cmake<C>(a0.x - (R)0.5 * s.x, a0.y - (R)0.5 * s.y);
    // +/- i*sign*h*d
    C t = cmake<C>(-(R)sign * h * d.y, (R)sign * h * d.x);
    b = cadd(m, t);
    c = csub(m, t);
}

// 4-point DFT of v[o], v[o+st], v[o+2st], v[o+3st] in place
template <typename C>
HPSI_D void dft4_at(C* v, int o, int st, int sign)
{
    C a0 = cadd(v[o], v[o + 2 * st]), a1 = csub(v[o], v[o + 2 * st]);
    C b0 = cadd(v[o + st], v[o + 3 * st]), b1 = cmul_i(csub(v[o + st], v[o + 3 * st]), sign);
    v[o] = cadd(a0, b0);
    v[o + 2 * st] = csub(a0, b0);
    v[o + st] = cadd(a1, b1);
    v[o + 3 * st] = csub(a1, b1);
}

// p-point DFT of v[0..p) in registers: v[q] <- sum_r v[r] W_p^{r q}
template <typename C, int P>
HPSI_D void dft_small(C (&v)[HPSI_FFT_MAXR], const C* tw, int n, int sign)
{
    using R = typename Real<C>::type;
    if constexpr (P == 3) {
        dft3(v[0], v[1], v[2], sign);
    } else if constexpr (P == 8) {
        // 8 = 2 x 4: x[2 n1 + n2]; inner 4-point DFTs over n1 (even / odd),
        // twiddle the odd one by W_8^{k1}, then 2-point DFTs
        C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        dft4_at(e, 0, 1, sign);
        dft4_at(o, 0, 1, sign);
        const R r2 = (R)0.70710678118654752440;
        // W_8^1 = (r2, sign r2), W_8^2 = sign i, W_8^3 = (-r2, sign r2)
        o[1] = cmul(o[1], cmake<C>(r2, (R)sign * r2));
        o[2] = cmul_i(o[2], sign);
        o[3] = cmul(o[3], cmake<C>(-r2, (R)sign * r2));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = cadd(e[k], o[k]);
            v[k + 4] = csub(e[k], o[k]);
        }
    } else if constexpr (P == 9) {
        // 9 = 3 x 3: x[3 n1 + n2]; inner 3-point DFTs over n1, twiddle by
        // W_9^{n2 k1}, then 3-point DFTs over n2; output index k1 + 3 k2
        C y[9];
#pragma unroll
        for (int n2 = 0; n2 < 3; ++n2) {
            C a = v[n2], b = v[3 + n2], c = v[6 + n2];
            dft3(a, b, c, sign);
            y[3 * n2] = a;
            y[3 * n2 + 1] = b;
            y[3 * n2 + 2] = c;
        }
        const int step = n / 9;
        y[4] = cmul(y[4], tw_get(tw, 1 * step, sign));
        y[5] = cmul(y[5], tw_get(tw, 2 * step, sign));
        y[7] = cmul(y[7], tw_get(tw, 2 * step, sign));
        y[8] = cmul(y[8], tw_get(tw, 4 * step, sign));
#pragma unroll
        for (int k1 = 0; k1 < 3; ++k1) {
            C a = y[k1], b = y[3 + k1], c = y[6 + k1];
            dft3(a, b, c, sign);
            v[k1] = a;
            v[k1 + 3] = b;
            v[k1 + 6] = c;
        }
    } else if constexpr (P == 2) {
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
// lines (use when ls == 1, or when the row stride ls is odd) or butterflies
// (use when es == 1), so that shared-memory accesses of a warp do not
// collide.  `nlf` divides by nl and `nsf` by Ns without integer division.
template <typename C, int P, bool LINE_FAST>
HPSI_D void fft_stage_p(const C* __restrict__ src, C* __restrict__ dst, int n, const FastDiv& nsf, const FastDiv& nlf,
                        int ls, int es, const C* tw, int sign)
{
    const int Ns = (int)nsf.d;
    const int nl = (int)nlf.d;
    const int nbf = n / P;
    const int total = nl * nbf;
    const int tstep = n / (Ns * P);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int L, i;
        if (LINE_FAST) { i = (int)fdiv((uint32_t)t, nlf); L = t - i * nl; }
        else { L = (int)(t / nbf); i = t - L * nbf; }
        const int hi = (int)fdiv((uint32_t)i, nsf);
        const int k = i - hi * Ns;
        const int tj = k * tstep;  // q * tj < n for q < P
        C v[HPSI_FFT_MAXR];
        const C* s = src + (size_t)L * ls;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            C x = s[(size_t)(i + q * nbf) * es];
            if (q > 0 && k > 0) x = cmul(x, tw_get(tw, q * tj, sign));
            v[q] = x;
        }
        dft_small<C, P>(v, tw, n, sign);
        C* d = dst + (size_t)L * ls;
        const int base = hi * Ns * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) d[(size_t)(base + q * Ns) * es] = v[q];
    }
}

// The same stage with element access through functors: ld(L, e) returns
// element e of line L, st(L, e, v) stores it.  Lets the first stage of a
// transform read straight from global memory and the last stage write straight
// to its destination (with any pointwise factor folded into st).
template <typename C, int P, bool LINE_FAST, typename LD, typename ST>
HPSI_D void fft_stage_io(const LD& ld, const ST& st, int n, const FastDiv& nsf, const FastDiv& nlf, const C* tw,
                         int sign)
{
    const int Ns = (int)nsf.d;
    const int nl = (int)nlf.d;
    const int nbf = n / P;
    const int total = nl * nbf;
    const int tstep = n / (Ns * P);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int L, i;
        if (LINE_FAST) { i = (int)fdiv((uint32_t)t, nlf); L = t - i * nl; }
        else { L = (int)(t / nbf); i = t - L * nbf; }
        const int hi = (int)fdiv((uint32_t)i, nsf);
        const int k = i - hi * Ns;
        const int tj = k * tstep;
        C v[HPSI_FFT_MAXR];
#pragma unroll
        for (int q = 0; q < P; ++q) v[q] = ld(L, i + q * nbf);
#pragma unroll
        for (int q = 1; q < P; ++q)
            if (k > 0) v[q] = cmul(v[q], tw_get(tw, q * tj, sign));
        dft_small<C, P>(v, tw, n, sign);
        const int base = hi * Ns * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) st(L, base + q * Ns, v[q]);
    }
}

// shared-memory line accessor: element e of line L at b[L*ls + e*es]
template <typename C>
struct SmemLines {
    C* b;
    int ls, es;
    HPSI_D C operator()(int L, int e) const { return b[L * ls + e * es]; }
    HPSI_D void operator()(int L, int e, C v) const { b[L * ls + e * es] = v; }
};

template <typename C, bool LINE_FAST, bool WIDE, typename LD, typename ST>
HPSI_D void fft_stage_io_p(int p, const LD& ld, const ST& st, int n, const FastDiv& nsf, const FastDiv& nlf,
                           const C* tw, int sign)
{
    switch (p) {
        case 8: fft_stage_io<C, 8, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        case 9: fft_stage_io<C, 9, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        case 2: fft_stage_io<C, 2, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        case 3: fft_stage_io<C, 3, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        case 4: fft_stage_io<C, 4, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        case 5: fft_stage_io<C, 5, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
        default:
            if constexpr (WIDE) {
                switch (p) {
                    case 7: fft_stage_io<C, 7, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
                    case 11: fft_stage_io<C, 11, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
                    case 13: fft_stage_io<C, 13, LINE_FAST>(ld, st, n, nsf, nlf, tw, sign); break;
                    default: break;
                }
            }
            break;
    }
}

// ---- compile-time two-stage transforms --------------------------------------
// For the grid lengths of the common cells (72 = 8*9, 36 = 9*4, 24 = 8*3,
// 64 = 8*8) the stage shapes are template constants: the per-element index
// arithmetic (butterfly -> group and offset, twiddle index, output position)
// folds into constant multiplies and shifts instead of runtime divisions.
// The radix order is the one fft_factor picks: the same arithmetic as the
// runtime-plan path.
template <int R0, int R1>
struct FftPlan2 {
    static constexpr int r0 = R0, r1 = R1, n = R0 * R1;
};

// Line accessor with compile-time strides: element e of line L at b[L*LS + e*ES]
template <typename C, int LS, int ES>
struct SmemLinesC {
    C* b;
    HPSI_D C operator()(int L, int e) const { return b[L * LS + e * ES]; }
    HPSI_D void operator()(int L, int e, C v) const { b[L * LS + e * ES] = v; }
};

// NLC > 0: the number of lines is the compile-time NLC, else nlf.d
template <typename C, int N, int P, int NS, int NLC, typename LD, typename ST>
HPSI_D void fft_stage_ct(const LD& ld, const ST& st, const FastDiv& nlf, const C* tw, int sign)
{
    constexpr int nbf = N / P;
    constexpr int tstep = N / (NS * P);
    const int nl = NLC > 0 ? NLC : (int)nlf.d;
    const int total = nl * nbf;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int i = NLC > 0 ? t / NLC : (int)fdiv((uint32_t)t, nlf);  // lines walked fastest
        const int L = t - i * nl;
        const int hi = i / NS;
        const int k = i - hi * NS;
        C v[HPSI_FFT_MAXR];
#pragma unroll
        for (int q = 0; q < P; ++q) v[q] = ld(L, i + q * nbf);
        if (NS > 1 && k > 0) {
#pragma unroll
            for (int q = 1; q < P; ++q) v[q] = cmul(v[q], tw_get(tw, q * k * tstep, sign));
        }
        dft_small<C, P>(v, tw, N, sign);
        const int base = hi * NS * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) st(L, base + q * NS, v[q]);
    }
}

// Two-stage transform of nl lines: stage 0 reads through ld and writes bufA
// (line stride ls, element stride es), stage 1 reads bufA and writes through
// st (the same buffer contract as fft_lines_io with nst == 2: the last stage
// reads bufA).
template <typename C, typename PL, typename LD, typename ST>
HPSI_D void fft_lines_ct(const LD& ld, const ST& st, C* bufA, const FastDiv& nlf, int ls, int es, const C* tw,
                         int sign)
{
    const SmemLines<C> A{bufA, ls, es};
    fft_stage_ct<C, PL::n, PL::r0, 1, 0>(ld, A, nlf, tw, sign);
    __syncthreads();
    fft_stage_ct<C, PL::n, PL::r1, PL::r0, 0>(A, st, nlf, tw, sign);
}

// The same with a compile-time line count NLC and intermediate accessor A
// (constant strides): no runtime index arithmetic left but the loop.
template <typename C, typename PL, int NLC, typename AB, typename LD, typename ST>
HPSI_D void fft_lines_cc(const LD& ld, const ST& st, const AB& A, const C* tw, int sign)
{
    const FastDiv unused{};
    fft_stage_ct<C, PL::n, PL::r0, 1, NLC>(ld, A, unused, tw, sign);
    __syncthreads();
    fft_stage_ct<C, PL::n, PL::r1, PL::r0, NLC>(A, st, unused, tw, sign);
}

// ---- pruned plane transforms --------------------------------------------
// A sphere plane holds G-vectors only in the rows j with |G_y| <= jr: rows
// 0..jr and n-jr..n-1.  The z-lines of the other rows are zero on input to
// G->r and not read after r->G, so these transforms visit the nl = 2 jr + 1
// rows in use: line L is row L (L <= jr) or row L + n - nl.
template <typename C, int LS, int ES>
struct SmemRowsC {
    C* b;
    int jr, gap;
    HPSI_D int row(int L) const { return L + (L > jr ? gap : 0); }
    HPSI_D C operator()(int L, int e) const { return b[row(L) * LS + e * ES]; }
    HPSI_D void operator()(int L, int e, C v) const { b[row(L) * LS + e * ES] = v; }
};

// fft_stage_ct with a run-time line count nl: t / nl from one multiply by
// rinv = 1/nl, exact for t < 2^12 and nl <= 2^8 (relative error of the
// product <= 2^-23, so the absolute error <= 2^-11 < 0.5 / nl, the distance
// of (t + 1/2) / nl from an integer)
template <typename C, int N, int P, int NS, typename LD, typename ST>
HPSI_D void fft_stage_rows(const LD& ld, const ST& st, int nl, float rinv, const C* tw, int sign)
{
    constexpr int nbf = N / P;
    constexpr int tstep = N / (NS * P);
    const int total = nl * nbf;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int i = (int)(((float)t + 0.5f) * rinv);
        const int L = t - i * nl;
        const int hi = i / NS;
        const int k = i - hi * NS;
        C v[HPSI_FFT_MAXR];
#pragma unroll
        for (int q = 0; q < P; ++q) v[q] = ld(L, i + q * nbf);
        if (NS > 1 && k > 0) {
#pragma unroll
            for (int q = 1; q < P; ++q) v[q] = cmul(v[q], tw_get(tw, q * k * tstep, sign));
        }
        dft_small<C, P>(v, tw, N, sign);
        const int base = hi * NS * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) st(L, base + q * NS, v[q]);
    }
}

// Two-stage transform of the rows in use (jr as above; 2 jr + 1 < n) of a
// plane with line stride LS and element stride ES: in -> A -> out (in may be out)
template <typename C, typename PL, int LS, int ES>
HPSI_D void fft_rows_cc(C* in, C* out, C* A, int jr, const C* tw, int sign)
{
    const int nl = 2 * jr + 1, gap = PL::n - nl;
    const float rinv = 1.0f / (float)nl;
    fft_stage_rows<C, PL::n, PL::r0, 1>(SmemRowsC<C, LS, ES>{in, jr, gap}, SmemRowsC<C, LS, ES>{A, jr, gap}, nl, rinv,
                                        tw, sign);
    __syncthreads();
    fft_stage_rows<C, PL::n, PL::r1, PL::r0>(SmemRowsC<C, LS, ES>{A, jr, gap}, SmemRowsC<C, LS, ES>{out, jr, gap}, nl,
                                             rinv, tw, sign);
}

// Plan ids the host selects (0 = runtime plan)
enum { FFT_CT_NONE = 0, FFT_CT_72 = 1, FFT_CT_36 = 2, FFT_CT_24 = 3, FFT_CT_64 = 4 };
static inline int fft_ct_id(const FftLen& L)
{
    if (L.nst != 2) return FFT_CT_NONE;
    if (L.rad[0] == 8 && L.rad[1] == 9) return FFT_CT_72;
    if (L.rad[0] == 9 && L.rad[1] == 4) return FFT_CT_36;
    if (L.rad[0] == 8 && L.rad[1] == 3) return FFT_CT_24;
    if (L.rad[0] == 8 && L.rad[1] == 8) return FFT_CT_64;
    return FFT_CT_NONE;
}

// Which buffer the last stage of fft_lines_io reads: 0 = ld, 1 = bufA, 2 = bufB.
HPSI_HD int fft_last_read(const FftLen& L) { return L.nst <= 1 ? 0 : (((L.nst - 2) % 2 == 0) ? 1 : 2); }

// Transform of nl lines: stage 0 reads through ld, the last stage writes
// through st, stages in between ping-pong through bufA (written by stages
// 0, 2, ...) and bufB (stages 1, 3, ...), laid out with line stride ls and
// element stride es.  ld must not read bufA.  A barrier separates stages; the
// caller synchronises after the last one.  Returns the buffer that the last
// stage read (so the caller may direct st to the other one): 0 = ld, 1 = bufA,
// 2 = bufB.
template <typename C, bool LINE_FAST, bool WIDE, typename LD, typename ST>
HPSI_D int fft_lines_io(const LD& ld, const ST& st, C* bufA, C* bufB, const FftLen& L, const FastDiv& nlf, int ls,
                        int es, const C* tw, int sign)
{
    if (L.nst == 0) {
        for (int t = threadIdx.x; t < (int)nlf.d; t += blockDim.x) st(t, 0, ld(t, 0));
        return 0;
    }
    const SmemLines<C> A{bufA, ls, es}, B{bufB, ls, es};
    for (int s = 0; s < L.nst; ++s) {
        const bool first = s == 0, last = s == L.nst - 1;
        const SmemLines<C>& in = ((s - 1) % 2 == 0) ? A : B;
        const SmemLines<C>& out = (s % 2 == 0) ? A : B;
        const int p = L.rad[s];
        if (first && last) fft_stage_io_p<C, LINE_FAST, WIDE>(p, ld, st, L.n, L.ns[s], nlf, tw, sign);
        else if (first) fft_stage_io_p<C, LINE_FAST, WIDE>(p, ld, out, L.n, L.ns[s], nlf, tw, sign);
        else if (last) fft_stage_io_p<C, LINE_FAST, WIDE>(p, in, st, L.n, L.ns[s], nlf, tw, sign);
        else fft_stage_io_p<C, LINE_FAST, WIDE>(p, in, out, L.n, L.ns[s], nlf, tw, sign);
        if (!last) __syncthreads();
    }
    return L.nst == 1 ? 0 : (((L.nst - 2) % 2 == 0) ? 1 : 2);
}

// Radices compiled into a stage: the narrow set {2,3,4,5,8,9} covers the
// usual 2^a 3^b 5^c grids with few registers; WIDE adds 7, 11 and 13.
template <typename C, bool LINE_FAST, bool WIDE>
HPSI_D void fft_stage(const C* src, C* dst, int p, int n, const FastDiv& nsf, const FastDiv& nlf, int ls, int es,
                      const C* tw, int sign)
{
    switch (p) {
        case 8: fft_stage_p<C, 8, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        case 9: fft_stage_p<C, 9, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        case 2: fft_stage_p<C, 2, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        case 3: fft_stage_p<C, 3, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        case 4: fft_stage_p<C, 4, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        case 5: fft_stage_p<C, 5, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
        default:
            if constexpr (WIDE) {
                switch (p) {
                    case 7: fft_stage_p<C, 7, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
                    case 11: fft_stage_p<C, 11, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
                    case 13: fft_stage_p<C, 13, LINE_FAST>(src, dst, n, nsf, nlf, ls, es, tw, sign); break;
                    default: break;
                }
            }
            break;  // fft_factor admits no other radix; the host picks WIDE when 7, 11 or 13 occur
    }
}

// true if a length needs the wide radix set
static inline bool fft_needs_wide(const FftLen& L)
{
    for (int s = 0; s < L.nst; ++s)
        if (L.rad[s] == 7 || L.rad[s] == 11 || L.rad[s] == 13) return true;
    return false;
}

// Full transform of the nl lines described by nlf; data starts in bufs[cur]
// and the function returns the index (0/1) of the buffer holding the result.
template <typename C, bool LINE_FAST, bool WIDE>
HPSI_D int fft_lines(C* buf0, C* buf1, int cur, const FftLen& L, const FastDiv& nlf, int ls, int es, const C* tw,
                     int sign)
{
    for (int s = 0; s < L.nst; ++s) {
        const int p = L.rad[s];
        C* src = cur ? buf1 : buf0;
        C* dst = cur ? buf0 : buf1;
        fft_stage<C, LINE_FAST, WIDE>(src, dst, p, L.n, L.ns[s], nlf, ls, es, tw, sign);
        __syncthreads();
        cur ^= 1;
    }
    return cur;
}
