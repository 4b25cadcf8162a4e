// common.cuh — complex helpers and launch utilities shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define HPSI_HD __host__ __device__ __forceinline__
#define HPSI_D __device__ __forceinline__

// Complex numbers are the CUDA vector types: double2 (complex128) and
// float2 (complex64), .x = real, .y = imaginary.  Real<T> maps a complex
// type to its scalar type.
template <typename C> struct Real;
template <> struct Real<double2> { using type = double; };
template <> struct Real<float2> { using type = float; };

template <typename C> HPSI_HD C cmake(typename Real<C>::type r, typename Real<C>::type i) { C c; c.x = r; c.y = i; return c; }
template <typename C> HPSI_HD C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> HPSI_HD C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> HPSI_HD C cmul(C a, C b) { return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C> HPSI_HD C cscale(C a, typename Real<C>::type s) { return cmake<C>(a.x * s, a.y * s); }
// multiply by +i (sign > 0) or -i (sign < 0)
template <typename C> HPSI_HD C cmul_i(C a, int sign) { return sign > 0 ? cmake<C>(-a.y, a.x) : cmake<C>(a.y, -a.x); }

// FP64 <-> FP32 conversions on the integer pipe.  GB300 executes FP64
// instructions, conversions included, at a small fraction of the FP32 rate;
// these use shifts and adds on the bit patterns instead.
//   d2f_bits: round to nearest even, exact for results in the normal float
//             range; overflow gives +-inf, NaN stays NaN; results below
//             2^-126 (float subnormals) flush to signed zero.
//   f2d_bits: exact for normal floats, inf and NaN; zero and subnormals give
//             signed zero.
#ifdef __CUDACC__
__device__ __forceinline__ float d2f_bits(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    // bits 31..23: the low 9 bits of the double exponent; 22..0: the top 23
    // mantissa bits.  Adding 2^30 rebiases the exponent (1023 -> 127) mod 2^9.
    uint32_t f = __funnelshift_l(lo, hi, 3) + 0x40000000u;
    // round half to even on the 29 dropped bits (a carry may bump the exponent)
    f += ((lo & 0x1fffffffu) + (f & 1u) + 0x0fffffffu) >> 29;
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const bool nan = e == 0x7ffu && (((hi & 0xfffffu) | lo) != 0u);
    f = e <= 896u ? 0u : (e >= 1151u ? (nan ? 0x7fc00000u : 0x7f800000u) : f);
    return __uint_as_float(f | (hi & 0x80000000u));
}

__device__ __forceinline__ double f2d_bits(float x)
{
    const uint32_t u = __float_as_uint(x), a = u & 0x7fffffffu;
    const bool normal = a >= 0x00800000u;
    uint32_t hi = normal ? (a >> 3) + 0x38000000u : 0u;  // exponent + (1023 - 127)
    if (a >= 0x7f800000u) hi = 0x7ff00000u | ((a >> 3) & 0xfffffu);  // inf, NaN
    const uint32_t lo = normal ? u << 29 : 0u;
    return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}
#endif

HPSI_HD float2 to_c64(double2 a)
{
#ifdef __CUDA_ARCH__
    return make_float2(d2f_bits(a.x), d2f_bits(a.y));
#else
    return make_float2((float)a.x, (float)a.y);
#endif
}
HPSI_HD double2 to_c128(float2 a)
{
#ifdef __CUDA_ARCH__
    return make_double2(f2d_bits(a.x), f2d_bits(a.y));
#else
    return make_double2((double)a.x, (double)a.y);
#endif
}
template <typename C> HPSI_HD C from_c128(double2 a);
template <> HPSI_HD double2 from_c128<double2>(double2 a) { return a; }
template <> HPSI_HD float2 from_c128<float2>(double2 a) { return to_c64(a); }
HPSI_HD double2 as_c128(double2 a) { return a; }
HPSI_HD double2 as_c128(float2 a) { return to_c128(a); }

#ifdef __CUDACC__
// Compensated FP32 sum (Knuth's two-sum): s + c carries about twice the
// precision of s alone, using the FP32 pipe only.
struct Sum2f {
    float s = 0.f, c = 0.f;
    HPSI_D void add(float x)
    {
        const float t = s + x, bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
    HPSI_D float value() const { return s + c; }
};
#endif

static inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }
