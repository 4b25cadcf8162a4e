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

HPSI_HD float2 to_c64(double2 a) { return make_float2((float)a.x, (float)a.y); }
HPSI_HD double2 to_c128(float2 a) { return make_double2((double)a.x, (double)a.y); }
template <typename C> HPSI_HD C from_c128(double2 a);
template <> HPSI_HD double2 from_c128<double2>(double2 a) { return a; }
template <> HPSI_HD float2 from_c128<float2>(double2 a) { return to_c64(a); }
HPSI_HD double2 as_c128(double2 a) { return a; }
HPSI_HD double2 as_c128(float2 a) { return to_c128(a); }

static inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }
