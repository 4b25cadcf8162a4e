// fft_reg.cuh — line transforms held entirely in one thread's registers.
//
// A line of N = N1*N2 complex64 values (N1, N2 in {3, 4, 8, 9}) lives in a
// register array v[N]; every index below is a compile-time constant, so the
// array stays in registers and the data movement between the two stages is
// register renaming: no shared memory, no barrier, no index arithmetic.
//
// Two orderings of the same transform (the index maps of the two-factor
// Cooley-Tukey split; S = +1 for G->r exp(+i..), -1 for r->G):
//
//   fft_nat_to_split<S, N1, N2>:  input natural, x[n] at v[n];
//     X[k1 + N1 k2] = sum_{n2} W_N^{S n2 k1} W_N2^{S n2 k2}
//                     sum_{n1} W_N1^{S n1 k1} x[N2 n1 + n2]
//     ends with X[k1 + N1 k2] at v[N2 k1 + k2].
//
//   fft_split_to_nat<S, N1, N2>:  input y[x1 + N1 x2] at v[N2 x1 + x2];
//     Y[N2 m1 + m2] = sum_{x1} W_N1^{S x1 m1} W_N^{S x1 m2}
//                     sum_{x2} W_N2^{S x2 m2} y[x1 + N1 x2]
//     ends natural, Y[m] at v[m].
//
// Applied back to back (G->r, a pointwise factor at the split positions,
// r->G) they give the x pass of the local term with no reordering at all.
// The transform conventions are the reference's FFT3D (src/math/fft.cppm:
// 18-85): G->r unnormalised with exp(+i...), r->G with exp(-i...); the 1/N
// normalisation is left to the caller.  Twiddles exp(2 pi i j/N) are
// compile-time constants (evaluated in double by the series below, rounded to
// float once), so they become instruction immediates.
#pragma once

#include "common.cuh"

namespace fftreg {

// ---- compile-time cos / sin of 2 pi j / n ---------------------------------
// Octant reduction with exact integer arithmetic, then Taylor series on
// [0, pi/4] in double (terms to x^27: error far below one double ulp there).
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double sin_poly(double x)
{
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / (double)((2 * k) * (2 * k + 1));
        sum += term;
    }
    return sum;
}

constexpr double cos_poly(double x)
{
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / (double)((2 * k - 1) * (2 * k));
        sum += term;
    }
    return sum;
}

// {cos, sin}(2 pi j / n) for any integer j, n > 0
struct CS {
    double c, s;
};
constexpr CS cossin_2pi(long j, long n)
{
    long a = ((j % n) + n) % n;  // 0 <= a < n; angle fraction t = a/n = num/(8n)
    long num = 8 * a;
    double sgn_s = 1.0, sgn_c = 1.0;
    bool swap = false;
    if (num > 4 * n) { num = 8 * n - num; sgn_s = -1.0; }  // t > 1/2: t -> 1 - t
    if (num > 2 * n) { num = 4 * n - num; sgn_c = -1.0; }  // t > 1/4: t -> 1/2 - t
    if (num > n) { num = 2 * n - num; swap = true; }       // t > 1/8: t -> 1/4 - t
    const double x = kPi * (double)num / (double)(4 * n);  // 2 pi t, in [0, pi/4]
    const double c0 = cos_poly(x), s0 = sin_poly(x);
    const double c = swap ? s0 : c0, s = swap ? c0 : s0;
    return CS{sgn_c * c, sgn_s * s};
}

// ---- complex helpers -------------------------------------------------------
// Complex adds and subtracts are packed FP32 pair operations (one instruction
// for the real and imaginary parts, each rounded as a scalar add): the
// transforms are issue-bound, and most of their instructions are these adds.
HPSI_D float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
HPSI_D float2 sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
// a * (S i)
template <int S>
HPSI_D float2 mul_si(float2 a)
{
    return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// a + S i d: scalar, the swapped components of i d need no pair of their own
template <int S>
HPSI_D float2 add_si(float2 a, float2 d)
{
    return S > 0 ? make_float2(a.x - d.y, a.y + d.x) : make_float2(a.x + d.y, a.y - d.x);
}

// a * exp(S 2 pi i J / N), J taken mod N; exact for the multiples of N/4
template <int N, int J, int S>
HPSI_D float2 twiddle(float2 a)
{
    constexpr int j = ((J % N) + N) % N;
    if constexpr (j == 0) {
        return a;
    } else if constexpr (4 * j == N) {
        return mul_si<S>(a);
    } else if constexpr (2 * j == N) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * j == 3 * N) {
        return mul_si<-S>(a);
    } else {
        constexpr CS w = cossin_2pi(j, N);
        constexpr float c = (float)w.c, s = (float)(S * w.s);
        return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
    }
}

// ---- small DFTs in place on v[B + k*ST], k < P (natural order out) --------
template <int S, int B, int ST, int N>
HPSI_D void dft2(float2 (&v)[N])
{
    const float2 a = v[B], b = v[B + ST];
    v[B] = add(a, b);
    v[B + ST] = sub(a, b);
}

template <int S, int B, int ST, int N>
HPSI_D void dft3(float2 (&v)[N])
{
    constexpr float h = 0.86602540378443864676f;  // sin(2 pi / 3)
    const float2 a = v[B], b = v[B + ST], c = v[B + 2 * ST];
    const float2 s = add(b, c), d = sub(b, c);
    const float2 m = __ffma2_rn(make_float2(-0.5f, -0.5f), s, a);
    const float2 hd = __fmul2_rn(make_float2(h, h), d);
    v[B] = add(a, s);
    v[B + ST] = add_si<S>(m, hd);   // m + S i h d
    v[B + 2 * ST] = add_si<-S>(m, hd);
}

template <int S, int B, int ST, int N>
HPSI_D void dft4(float2 (&v)[N])
{
    const float2 y0 = v[B], y1 = v[B + ST], y2 = v[B + 2 * ST], y3 = v[B + 3 * ST];
    const float2 t0 = add(y0, y2), t1 = sub(y0, y2), t2 = add(y1, y3), d = sub(y1, y3);
    v[B] = add(t0, t2);
    v[B + 2 * ST] = sub(t0, t2);
    v[B + ST] = add_si<S>(t1, d);       // t1 + S i d
    v[B + 3 * ST] = add_si<-S>(t1, d);  // t1 - S i d
}

// 8 = 2 x 4: 4-point DFTs of the even and odd elements, W_8^k on the odd ones
template <int S, int B, int ST, int N>
HPSI_D void dft8(float2 (&v)[N])
{
    float2 e[4] = {v[B], v[B + 2 * ST], v[B + 4 * ST], v[B + 6 * ST]};
    float2 o[4] = {v[B + ST], v[B + 3 * ST], v[B + 5 * ST], v[B + 7 * ST]};
    dft4<S, 0, 1>(e);
    dft4<S, 0, 1>(o);
    constexpr float r2 = 0.70710678118654752440f;
    o[1] = make_float2(r2 * (o[1].x - S * o[1].y), r2 * (S * o[1].x + o[1].y));    // * (r2, S r2)
    o[3] = make_float2(-r2 * (o[3].x + S * o[3].y), r2 * (S * o[3].x - o[3].y));   // * (-r2, S r2)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k == 2) {  // * S i
            v[B + k * ST] = add_si<S>(e[k], o[k]);
            v[B + (k + 4) * ST] = add_si<-S>(e[k], o[k]);
        } else {
            v[B + k * ST] = add(e[k], o[k]);
            v[B + (k + 4) * ST] = sub(e[k], o[k]);
        }
    }
}

// 9 = 3 x 3: x[3 n1 + n2]; 3-point DFTs over n1, W_9^{n2 k1}, 3-point DFTs
// over n2; X[k1 + 3 k2]
template <int S, int B, int ST, int N>
HPSI_D void dft9(float2 (&v)[N])
{
    float2 y[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) y[i] = v[B + i * ST];
    dft3<S, 0, 3>(y);  // n2 = 0: y[0], y[3], y[6] -> k1 = 0, 1, 2
    dft3<S, 1, 3>(y);
    dft3<S, 2, 3>(y);
    // y[3 k1 + n2] now holds the k1 output of column n2
    y[4] = twiddle<9, 1, S>(y[4]);
    y[5] = twiddle<9, 2, S>(y[5]);
    y[7] = twiddle<9, 2, S>(y[7]);
    y[8] = twiddle<9, 4, S>(y[8]);
    dft3<S, 0, 1>(y);  // k1 = 0: y[0..2] over n2 -> k2
    dft3<S, 3, 1>(y);
    dft3<S, 6, 1>(y);
    // y[3 k1 + k2] = X[k1 + 3 k2]
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 3; ++k2) v[B + (k1 + 3 * k2) * ST] = y[3 * k1 + k2];
}

template <int P, int S, int B, int ST, int N>
HPSI_D void dft(float2 (&v)[N])
{
    static_assert(P == 2 || P == 3 || P == 4 || P == 8 || P == 9, "radix");
    if constexpr (P == 2) dft2<S, B, ST>(v);
    else if constexpr (P == 3) dft3<S, B, ST>(v);
    else if constexpr (P == 4) dft4<S, B, ST>(v);
    else if constexpr (P == 8) dft8<S, B, ST>(v);
    else dft9<S, B, ST>(v);
}

// ---- the two orderings of the N1 x N2 transform ----------------------------
template <int S, int N1, int N2, int I, int N>
HPSI_D void cols_n1(float2 (&v)[N])  // DFT_N1 over v[N2 n1 + I], I < N2
{
    if constexpr (I < N2) {
        dft<N1, S, I, N2>(v);
        cols_n1<S, N1, N2, I + 1>(v);
    }
}

template <int S, int N1, int N2, int I, int N>
HPSI_D void rows_n2(float2 (&v)[N])  // DFT_N2 over v[N2 I + n2], I < N1
{
    if constexpr (I < N1) {
        dft<N2, S, N2 * I, 1>(v);
        rows_n2<S, N1, N2, I + 1>(v);
    }
}

template <int S, int N1, int N2, int R, int C, int N>
HPSI_D void twiddle_grid(float2 (&v)[N])  // v[N2 r + c] *= W_N^{S r c}
{
    if constexpr (R < N1) {
        if constexpr (C < N2) {
            v[N2 * R + C] = twiddle<N1 * N2, R * C, S>(v[N2 * R + C]);
            twiddle_grid<S, N1, N2, R, C + 1>(v);
        } else {
            twiddle_grid<S, N1, N2, R + 1, 0>(v);
        }
    }
}

template <int S, int N1, int N2>
HPSI_D void fft_nat_to_split(float2 (&v)[N1 * N2])
{
    cols_n1<S, N1, N2, 0>(v);          // output k1 of column n2 at N2 k1 + n2
    twiddle_grid<S, N1, N2, 0, 0>(v);  // W_N^{S k1 n2}
    rows_n2<S, N1, N2, 0>(v);          // output k2 of row k1 at N2 k1 + k2
}

template <int S, int N1, int N2>
HPSI_D void fft_split_to_nat(float2 (&v)[N1 * N2])
{
    rows_n2<S, N1, N2, 0>(v);          // over x2: m2 of row x1 at N2 x1 + m2
    twiddle_grid<S, N1, N2, 0, 0>(v);  // W_N^{S x1 m2}
    cols_n1<S, N1, N2, 0>(v);          // over x1: m1 at N2 m1 + m2 = m
}

// position in v of natural index x after fft_nat_to_split: x = k1 + N1 k2 -> N2 k1 + k2
template <int N1, int N2>
HPSI_HD constexpr int split_pos(int x)
{
    return N2 * (x % N1) + x / N1;
}

// ---- a line of N = 2 H on a lane pair ------------------------------------
// Lanes l and l ^ 16 of a warp share one line (the "even" lane is the one in
// the lower half-warp), so that each half-warp touches 16 consecutive lines
// or elements: coalesced global accesses and conflict-free shared-memory rows
// and columns.  Half the registers of a one-thread line; every lane of the
// warp must make the calls (the exchange is a full-warp shuffle).
//
// fft_pair (decimation in time): the even lane holds x[2n], the odd lane
// x[2n+1] (n < H = N1 N2, natural order in v).  Each lane transforms its half
// in registers, the odd lane multiplies by W_N^{S m}, and one exchange gives
//   even lane:  X[m]     = E[m] + W_N^{S m} O[m]
//   odd lane:   X[m + H] = E[m] - W_N^{S m} O[m],   m < H,
// with X[m (+ H)] left at v[split_pos<N1, N2>(m)].

template <int S, int N1, int N2, int I>
HPSI_D void pair_twiddle(float2 (&v)[N1 * N2])  // v[split_pos(m)] *= W_{2H}^{S m}, m = I..H-1
{
    constexpr int H = N1 * N2;
    if constexpr (I < H) {
        constexpr int r = split_pos<N1, N2>(I);
        v[r] = twiddle<2 * H, I, S>(v[r]);
        pair_twiddle<S, N1, N2, I + 1>(v);
    }
}

// even lane: v + partner's v; odd lane: partner's v - v
template <int H>
HPSI_D void pair_exchange(float2 (&v)[H], bool odd)
{
    const float sgn = odd ? -1.f : 1.f;
#pragma unroll
    for (int r = 0; r < H; ++r) {
        const float ox = __shfl_xor_sync(0xffffffffu, v[r].x, 16);
        const float oy = __shfl_xor_sync(0xffffffffu, v[r].y, 16);
        v[r] = make_float2(fmaf(sgn, v[r].x, ox), fmaf(sgn, v[r].y, oy));
    }
}

// half-length plans H = h1 h2 of the lane-pair transforms of the common lines
template <int N> struct PairPlan;
template <> struct PairPlan<72> { static constexpr int h1 = 9, h2 = 4; };
template <> struct PairPlan<36> { static constexpr int h1 = 9, h2 = 2; };
template <> struct PairPlan<24> { static constexpr int h1 = 4, h2 = 3; };
template <> struct PairPlan<64> { static constexpr int h1 = 8, h2 = 4; };

template <int S, int N1, int N2>
HPSI_D void fft_pair(float2 (&v)[N1 * N2], bool odd)
{
    fft_nat_to_split<S, N1, N2>(v);
    if (odd) pair_twiddle<S, N1, N2, 0>(v);
    pair_exchange<N1 * N2>(v, odd);
}

}  // namespace fftreg

