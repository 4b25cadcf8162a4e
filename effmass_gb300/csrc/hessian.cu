// hessian.cu — second k-derivatives of the projectors for d2H/dk_a dk_b |psi>
// (hpsi_hess_apply).  The reference declares the Hessian operator and its six
// outputs (src/H_psi/hamiltonian.cppm:84-91) but leaves it empty
// (src/H_psi/hamiltonian_hessian.cpp:48-50); this is the project's own.
//
// A projector's K-dependence is u(K) = beta(q) Y_lm(K^) = F0(q) R_lm(K), with
// R_lm = |K|^l Y_lm the real solid harmonic (a homogeneous polynomial,
// solid_harmonics.inc) and F0 = beta / q^l.  With g_n(x) = j_n(x) / x^n and
//   F0(q) =  4 pi Int beta r^(l+1) g_l(q r) dr
//   F1(q) = -4 pi Int beta r^(l+3) g_(l+1)(q r) dr      (= F0'(q) / q)
//   F3(q) =  4 pi Int beta r^(l+5) g_(l+2)(q r) dr      (= (F0'' - F0'/q) / q^2)
// every derivative is smooth, q = 0 included:
//   d_a u    = F1 K_a R + F0 d_a R
//   d_ab u   = F3 K_a K_b R + F1 (delta_ab R + K_a d_b R + K_b d_a R) + F0 d_ab R.
// The tables are built here from the radial projectors (Simpson rule as the
// reference's, numerical.cppm:33-90) and interpolated with its 4-point
// Lagrange stencil; the structure factor multiplies as for the projectors
// (its k-dependent phase is common to an atom's projectors and cancels in
// |p><p|, as in the reference's gradient).
#include "kernels.cuh"
#include "solid_harmonics.inc"

namespace {

// g_n(x) = j_n(x) / x^n: power series below x = n + 2 (no cancellation), else
// j_0, j_1 in closed form, the upward recurrence (stable for x > n) and x^-n
__device__ double gn(int n, double x)
{
    if (x < n + 2.0) {
        const double x2h = x * x / 2.0;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k <= 80; ++k) {
            term *= -x2h / ((double)k * (2.0 * n + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-17 * fabs(sum)) break;
        }
        double df = 1.0;
        for (int i = 3; i <= 2 * n + 1; i += 2) df *= i;
        return sum / df;
    }
    double s, c;
    sincos(x, &s, &c);
    double jp = s / x, jc = jp / x - c / x;  // j0, j1
    if (n == 0) return jp;
    for (int m = 1; m < n; ++m) {
        const double jn = (2.0 * m + 1.0) / x * jc - jp;
        jp = jc;
        jc = jn;
    }
    double xn = 1.0;
    for (int i = 0; i < n; ++i) xn *= x;
    return jc / xn;
}

__device__ double simpson_wt(int i, int n, bool uniform, const double* rab)
{
    const double h = uniform ? rab[0] : rab[i];
    if (n == 1) return h;
    if (n % 2 == 1) return ((i == 0 || i == n - 1) ? 1.0 : (i % 2 == 0 ? 2.0 : 4.0)) * h / 3.0;
    if (n == 2) return 0.5 * h;
    double w = 0.0;
    if (i <= 3) w += (i == 0 || i == 3 ? 1.0 : 3.0) * (3.0 / 8.0);
    if (i == 3) w += 1.0 / 3.0;
    if (i == n - 1) w += 1.0 / 3.0;
    else if (i >= 4) w += (i % 2 == 0 ? 4.0 : 2.0) / 3.0;
    return w * h;
}

// f[t][p][iq], t = 0, 1, 2 for F0, F1, F3; one block per (q, projector)
__global__ void __launch_bounds__(128) hess_table_kernel(int nr, const double* __restrict__ r,
                                                         const double* __restrict__ rab, int uniform,
                                                         const int* __restrict__ l_of, const int* __restrict__ nmax,
                                                         const double* __restrict__ beta, double dq, int nq, int np,
                                                         double* __restrict__ f)
{
    __shared__ double red[3][4];
    const int iq = blockIdx.x, p = blockIdx.y, l = l_of[p], n = nmax[p];
    const double q = iq * dq;
    const double* b = beta + (size_t)p * nr;
    double s0 = 0.0, s1 = 0.0, s3 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double ri = r[i], x = q * ri;
        double rl = 1.0;
        for (int k = 0; k < l; ++k) rl *= ri;
        const double w = simpson_wt(i, n, uniform != 0, rab) * b[i] * rl * ri;  // beta r^(l+1)
        s0 += w * gn(l, x);
        s1 += w * ri * ri * gn(l + 1, x);
        s3 += w * ri * ri * ri * ri * gn(l + 2, x);
    }
    double v[3] = {s0, s1, s3};
    for (int t = 0; t < 3; ++t) {
        double a = v[t];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) red[t][threadIdx.x >> 5] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double FOUR_PI = 4.0 * 3.14159265358979323846;
        const double sign[3] = {1.0, -1.0, 1.0};
        for (int t = 0; t < 3; ++t)
            f[((size_t)t * np + p) * nq + iq] = sign[t] * FOUR_PI * (red[t][0] + red[t][1] + red[t][2] + red[t][3]);
    }
}

// the reference's 4-point Lagrange interpolation (numerical.cppm:93-104) on a table t[nq]
__device__ double lag4(const double* t, int nq, double dq, double q)
{
    const double s = q / dq;
    int i0 = (int)floor(s) - 1;
    double px = s - i0;
    if (i0 < 0) { i0 = 0; px = s; }
    if (i0 + 3 >= nq) i0 = nq - 4;
    const double ux = 1.0 - px, vx = 2.0 - px, wx = 3.0 - px;
    return t[i0] * ux * vx * wx / 6.0 + t[i0 + 1] * px * vx * wx / 2.0 - t[i0 + 2] * px * ux * wx / 2.0 +
           t[i0 + 3] * px * ux * vx / 6.0;
}

__device__ __forceinline__ double ipow(double x, int n)
{
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

// second-derivative rows: d2[c][row][g], c = xx, yy, zz, xy, xz, yz
template <typename C>
__global__ void hess_assemble_kernel(int P, int npw, const ProjRow* __restrict__ rows,
                                     const double* __restrict__ ftabs, int nq, double dq, double inv_sqrt_omega,
                                     const double* __restrict__ kvec, const double2* __restrict__ sf,
                                     C* __restrict__ d2)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)P * npw) return;
    const int row = (int)(i / npw), g = (int)(i - (size_t)row * npw);
    const ProjRow pr = rows[row];
    const double K[3] = {kvec[3 * g], kvec[3 * g + 1], kvec[3 * g + 2]};
    const double q = sqrt(K[0] * K[0] + K[1] * K[1] + K[2] * K[2]);
    // radial tables of this radial function: [3][nq]
    const double* ft = ftabs + (size_t)pr.rad * 3 * nq;
    const double F0 = lag4(ft, nq, dq, q) * inv_sqrt_omega;
    const double F1 = lag4(ft + nq, nq, dq, q) * inv_sqrt_omega;
    const double F3 = lag4(ft + 2 * nq, nq, dq, q) * inv_sqrt_omega;
    // solid harmonic, its gradient and Hessian
    const int lm = pr.l * pr.l + pr.l + pr.m;
    double R = 0.0, dR[3] = {0, 0, 0}, H[6] = {0, 0, 0, 0, 0, 0};
    for (int t = 0; t < kShCount[lm]; ++t) {
        const ShTerm s = kSh[lm][t];
        const int e[3] = {s.a, s.b, s.z};
        R += s.c * ipow(K[0], e[0]) * ipow(K[1], e[1]) * ipow(K[2], e[2]);
        for (int a = 0; a < 3; ++a) {
            if (e[a] == 0) continue;
            int f[3] = {e[0], e[1], e[2]};
            f[a] -= 1;
            dR[a] += s.c * e[a] * ipow(K[0], f[0]) * ipow(K[1], f[1]) * ipow(K[2], f[2]);
        }
        const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
        for (int c = 0; c < 6; ++c) {
            int f[3] = {e[0], e[1], e[2]};
            double coef = s.c * f[pa[c]];
            f[pa[c]] -= 1;
            coef *= f[pb[c]];
            f[pb[c]] -= 1;
            if (coef != 0.0 && f[0] >= 0 && f[1] >= 0 && f[2] >= 0)
                H[c] += coef * ipow(K[0], f[0]) * ipow(K[1], f[1]) * ipow(K[2], f[2]);
        }
    }
    const double2 S = sf[(size_t)pr.atom * npw + g];
    const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    for (int c = 0; c < 6; ++c) {
        const int a = pa[c], b = pb[c];
        const double u = F3 * K[a] * K[b] * R + F1 * ((a == b ? R : 0.0) + K[a] * dR[b] + K[b] * dR[a]) + F0 * H[c];
        d2[((size_t)c * P + row) * npw + g] = from_c128<C>(make_double2(u * S.x, u * S.y));
    }
}

// out_b += psi_b (the kinetic Hessian delta_ab for a == b)
__global__ void add_kernel(size_t n, const double2* __restrict__ x, double2* __restrict__ y)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        y[i].x += x[i].x;
        y[i].y += x[i].y;
    }
}

}  // namespace

cudaError_t launch_hess_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                               const int* nmax, const double* beta, double dq, int nq, double* f, cudaStream_t st)
{
    if (np == 0 || nq == 0) return cudaSuccess;
    hess_table_kernel<<<dim3(nq, np), 128, 0, st>>>(nr, r, rab, uniform, l, nmax, beta, dq, nq, np, f);
    return cudaGetLastError();
}

template <typename C>
cudaError_t launch_hess_assemble(int P, int npw, const ProjRow* rows, const double* ftabs, int nq, double dq,
                                 double inv_sqrt_omega, const double* kvec, const double2* sf, C* d2, cudaStream_t st)
{
    const size_t n = (size_t)P * npw;
    if (n == 0) return cudaSuccess;
    hess_assemble_kernel<C><<<ceil_div((long)n, 128), 128, 0, st>>>(P, npw, rows, ftabs, nq, dq, inv_sqrt_omega, kvec,
                                                                     sf, d2);
    return cudaGetLastError();
}

cudaError_t launch_add(size_t n, const double2* x, double2* y, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    add_kernel<<<ceil_div((long)n, 256), 256, 0, st>>>(n, x, y);
    return cudaGetLastError();
}

template cudaError_t launch_hess_assemble<double2>(int, int, const ProjRow*, const double*, int, double, double,
                                                   const double*, const double2*, double2*, cudaStream_t);
template cudaError_t launch_hess_assemble<float2>(int, int, const ProjRow*, const double*, int, double, double,
                                                  const double*, const double2*, float2*, cudaStream_t);
