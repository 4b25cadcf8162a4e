// tables.cu — beta(q) and dbeta/dq tables of the radial projectors on the
// device (hpsi_beta_tables), so that a context can be set up from the radial
// pseudopotential data without a host quadrature.
//
// Reference: BetaqTables / DBetaqTables (src/pseudo/ncpp_advance.cppm:524-641,
// 718-835): on q_i = i dq, i < ceil(q_max/dq) + 4,
//   beta_q  = 4 pi Simpson[ beta(r) r   j_l(q r) ]
//   dbeta_q = 4 pi Simpson[ beta(r) r^2 j_l'(q r) ],  j_l' = (l/x) j_l - j_{l+1},
// each projector's trailing zeros trimmed, Simpson as src/math/numerical.cppm:33-90
// (3/8 rule on the first four points and 1/3 on the rest for an even count).
// j_l(x) is evaluated as the reference's SphericalBesselJ produces it
// (src/math/sph_bessel.cppm): the power series below x = 0.5, else j_0 and j_1
// in closed form and the upward recurrence.  One block per (q, projector);
// the Simpson sum is a weighted FP64 block reduction.
#include "kernels.cuh"

namespace {

__device__ double jl_ref(int l, double x)
{
    if (x < 1e-15) return l == 0 ? 1.0 : 0.0;
    if (x < 0.5) {
        const double x2h = x * x / 2.0;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k <= 50; ++k) {
            term *= -x2h / ((double)k * (2.0 * l + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-16 * fabs(sum)) break;
        }
        double df = 1.0, xl = 1.0;
        for (int i = 3; i <= 2 * l + 1; i += 2) df *= i;
        for (int i = 0; i < l; ++i) xl *= x;
        return sum * xl / df;
    }
    double s, c;
    sincos(x, &s, &c);
    const double j0 = s / x;
    if (l == 0) return j0;
    const double j1 = j0 / x - c / x;
    double jp = j0, jc = j1;
    for (int n = 1; n < l; ++n) {
        const double jn = (2.0 * n + 1.0) / x * jc - jp;
        jp = jc;
        jc = jn;
    }
    return jc;
}

// Simpson weight of point i of n (times rab[i] on a general mesh, rab[0] on a uniform one)
__device__ double simpson_w(int i, int n, bool uniform, const double* rab)
{
    const double h = uniform ? rab[0] : rab[i];
    if (n == 1) return h;
    if (n % 2 == 1) {
        const double w = (i == 0 || i == n - 1) ? 1.0 : (i % 2 == 0 ? 2.0 : 4.0);
        return w * h / 3.0;
    }
    if (n == 2) return 0.5 * h;
    // 3/8 on points 0..3; 1/3 rule from point 3 to n-1 (point 3 and n-1 are its ends,
    // counted twice when n == 4, as the reference's sum13 = f[3] + f[n-1] does)
    double w = 0.0;
    if (i <= 3) w += (i == 0 || i == 3 ? 1.0 : 3.0) * (3.0 / 8.0);
    if (i == 3) w += 1.0 / 3.0;
    if (i == n - 1) w += 1.0 / 3.0;
    else if (i >= 4) w += (i % 2 == 0 ? 4.0 : 2.0) / 3.0;
    return w * h;
}

__device__ __forceinline__ double block_sum_t(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red[w];
    return r;
}

__global__ void __launch_bounds__(128) beta_table_kernel(int nr, const double* __restrict__ r,
                                                         const double* __restrict__ rab, int uniform,
                                                         const int* __restrict__ l_of, const int* __restrict__ nmax,
                                                         const double* __restrict__ beta, double dq, int nq,
                                                         double* __restrict__ bq, double* __restrict__ dbq)
{
    __shared__ double red[8];
    const int iq = blockIdx.x, p = blockIdx.y, l = l_of[p], n = nmax[p];
    const double q = iq * dq;
    const double* b = beta + (size_t)p * nr;
    double s0 = 0.0, s1 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double x = q * r[i];
        const double w = simpson_w(i, n, uniform != 0, rab) * b[i] * r[i];
        const double jl = jl_ref(l, x);
        s0 += w * jl;
        if (dbq) {
            const double d = x < 1e-15 ? (l == 1 ? 1.0 / 3.0 : 0.0) : (double)l / x * jl - jl_ref(l + 1, x);
            s1 += w * r[i] * d;
        }
    }
    const double FOUR_PI = 4.0 * 3.14159265358979323846;
    const double t0 = block_sum_t(s0, red);
    __syncthreads();
    const double t1 = block_sum_t(s1, red);
    if (threadIdx.x == 0) {
        bq[(size_t)p * nq + iq] = FOUR_PI * t0;
        if (dbq) dbq[(size_t)p * nq + iq] = FOUR_PI * t1;
    }
}

// nmax[p] = 1 + index of the last non-zero beta_p(r_i) (0 if all zero)
__global__ void __launch_bounds__(128) trim_kernel(int nr, const double* __restrict__ beta, int* __restrict__ nmax)
{
    __shared__ int red[4];
    const double* b = beta + (size_t)blockIdx.x * nr;
    int m = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x)
        if (b[i] != 0.0) m = max(m, i + 1);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) nmax[blockIdx.x] = max(max(red[0], red[1]), max(red[2], red[3]));
}

}  // namespace

cudaError_t launch_trim(int nr, int np, const double* beta, int* nmax, cudaStream_t st)
{
    if (np == 0) return cudaSuccess;
    trim_kernel<<<np, 128, 0, st>>>(nr, beta, nmax);
    return cudaGetLastError();
}

int beta_table_nq(double dq, double q_max) { return (int)ceil(q_max / dq) + 1 + 3; }

cudaError_t launch_beta_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                               const int* nmax, const double* beta, double dq, int nq, double* bq, double* dbq,
                               cudaStream_t st)
{
    if (np == 0 || nq == 0) return cudaSuccess;
    beta_table_kernel<<<dim3(nq, np), 128, 0, st>>>(nr, r, rab, uniform, l, nmax, beta, dq, nq, bq, dbq);
    return cudaGetLastError();
}

// ---- G-sphere of a k-point on the device (hpsi_gsphere) ----------------------
// All integer G in the box |g_d| <= gmax with |k+G|^2/2 < ecut, K = (k+g) B
// (B rows = reciprocal vectors), in lexicographic (g1, g2, g3) order: a count
// pass per g1-plane, then one block per plane writes its points in order
// with a block-wide prefix over (g2, g3).
namespace {

struct GsArgs {
    double B[9];
    double kf[3];
    double ecut;
    int gmax;
};

__device__ __forceinline__ void gs_point(const GsArgs& a, int g1, int g2, int g3, double* K, double* kin)
{
    const double f0 = g1 + a.kf[0], f1 = g2 + a.kf[1], f2 = g3 + a.kf[2];
    K[0] = f0 * a.B[0] + f1 * a.B[3] + f2 * a.B[6];
    K[1] = f0 * a.B[1] + f1 * a.B[4] + f2 * a.B[7];
    K[2] = f0 * a.B[2] + f1 * a.B[5] + f2 * a.B[8];
    *kin = 0.5 * (K[0] * K[0] + K[1] * K[1] + K[2] * K[2]);
}

__global__ void __launch_bounds__(256) gs_count_kernel(GsArgs a, int* __restrict__ counts)
{
    __shared__ int red[8];
    const int L = 2 * a.gmax + 1, g1 = (int)blockIdx.x - a.gmax;
    int c = 0;
    for (int p = threadIdx.x; p < L * L; p += blockDim.x) {
        double K[3], kin;
        gs_point(a, g1, p / L - a.gmax, p % L - a.gmax, K, &kin);
        c += kin < a.ecut;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < 8; ++w) s += red[w];
        counts[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) gs_write_kernel(GsArgs a, const int* __restrict__ offsets, int* __restrict__ g,
                                                       double* __restrict__ kvec, double* __restrict__ kinetic)
{
    __shared__ int wsum[8];
    __shared__ int base;
    const int L = 2 * a.gmax + 1, g1 = (int)blockIdx.x - a.gmax;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) base = offsets[blockIdx.x];
    __syncthreads();
    for (int p0 = 0; p0 < L * L; p0 += blockDim.x) {
        const int p = p0 + threadIdx.x;
        double K[3], kin = 0.0;
        bool in = false;
        if (p < L * L) {
            gs_point(a, g1, p / L - a.gmax, p % L - a.gmax, K, &kin);
            in = kin < a.ecut;
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (lane == 0) wsum[warp] = __popc(m);
        __syncthreads();
        int before = base;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        if (in) {
            const int pos = before + __popc(m & ((1u << lane) - 1u));
            g[3 * pos] = g1;
            g[3 * pos + 1] = p / L - a.gmax;
            g[3 * pos + 2] = p % L - a.gmax;
            kvec[3 * pos] = K[0];
            kvec[3 * pos + 1] = K[1];
            kvec[3 * pos + 2] = K[2];
            kinetic[pos] = kin;
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < 8; ++w) base += wsum[w];
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_gs_count(const double* B, const double* kf, double ecut, int gmax, int* counts, cudaStream_t st)
{
    GsArgs a;
    for (int i = 0; i < 9; ++i) a.B[i] = B[i];
    for (int i = 0; i < 3; ++i) a.kf[i] = kf[i];
    a.ecut = ecut;
    a.gmax = gmax;
    gs_count_kernel<<<2 * gmax + 1, 256, 0, st>>>(a, counts);
    return cudaGetLastError();
}

cudaError_t launch_gs_write(const double* B, const double* kf, double ecut, int gmax, const int* offsets, int* g,
                            double* kvec, double* kinetic, cudaStream_t st)
{
    GsArgs a;
    for (int i = 0; i < 9; ++i) a.B[i] = B[i];
    for (int i = 0; i < 3; ++i) a.kf[i] = kf[i];
    a.ecut = ecut;
    a.gmax = gmax;
    gs_write_kernel<<<2 * gmax + 1, 256, 0, st>>>(a, offsets, g, kvec, kinetic);
    return cudaGetLastError();
}
