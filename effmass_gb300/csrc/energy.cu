// energy.cu — FP64 band-energy reductions <psi_b|H|psi_b> beside a mixed-
// precision H|psi> (hpsi_apply_energies).
//
// The reference forms band energies as Rayleigh quotients of H|psi> on the
// host (test/H_psi/test_hpsi_eigen.cpp:92-106).  Here every sum is FP64 and
// taken on the device from the quantities the H|psi> launches already hold:
//   kinetic   sum_G kinetic(G) |psi(G)|^2                         (exact inputs)
//   local     (1/N) sum_r V(r) |psi(r)|^2, from the x pass's FP64 sums
//             S1 = sum_r V |psi_32(r)|^2 and S0 = sum_r |psi_32(r)|^2 of the
//             complex64 transform, as S1 / S0 * sum_G |psi(G)|^2 (Parseval:
//             S0 = N sum_G |psi|^2 in exact arithmetic, so the transform's
//             gain error cancels; every G-vector has its own grid point)
//   nonlocal  sum_p lambda_p |<p|psi>|^2 from the projection's split-K
//             partial sums.
// All reductions run in a fixed order (one block per band, tree in shared
// memory), so results are reproducible bit for bit.
#include "kernels.cuh"

namespace {

__device__ __forceinline__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// out[b] = {sum_G kinetic |psi|^2, sum_G |psi|^2} in G order (coalesced); used
// when every G-vector has its own grid point
// Grid (nb, KN_CHUNKS): chunk c of band b writes out[(b * KN_CHUNKS + c) * 2 + {0, 1}].
constexpr int KN_CHUNKS = 8;
__global__ void __launch_bounds__(256) kin_norm_kernel(int npw, const double2* __restrict__ psi,
                                                       const double* __restrict__ kinetic, double* __restrict__ out)
{
    __shared__ double red[32];
    const double2* p = psi + (size_t)blockIdx.x * npw;
    const int per = (npw + KN_CHUNKS - 1) / KN_CHUNKS;
    const int g0 = blockIdx.y * per, g1 = min(npw, g0 + per);
    double k = 0.0, n = 0.0;
    for (int g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
        const double2 v = p[g];
        const double m = v.x * v.x + v.y * v.y;
        k += kinetic[g] * m;
        n += m;
    }
    k = block_sum(k, red);
    n = block_sum(n, red);
    if (threadIdx.x == 0) {
        out[2 * (blockIdx.x * KN_CHUNKS + blockIdx.y)] = k;
        out[2 * (blockIdx.x * KN_CHUNKS + blockIdx.y) + 1] = n;
    }
}

// out[b] = {S1, S0} summed over the x-pass slots of band b
__global__ void __launch_bounds__(256) local_sums_kernel(int nslots, const double* __restrict__ epart,
                                                         double* __restrict__ out)
{
    __shared__ double red[32];
    const double* e = epart + (size_t)blockIdx.x * nslots * 2;
    double s1 = 0.0, s0 = 0.0;
    for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
        s1 += e[2 * i];
        s0 += e[2 * i + 1];
    }
    s1 = block_sum(s1, red);
    s0 = block_sum(s0, red);
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = s1;
        out[2 * blockIdx.x + 1] = s0;
    }
}

// out[b] = sum_p lam_p |sum_s part[s][p][b]|^2  (SIMT projection partials)
template <typename Acc>
__global__ void __launch_bounds__(256) nl_energy_kernel(int P, int nb, int nsplit, const Acc* __restrict__ part,
                                                        const double* __restrict__ lam, double* __restrict__ out)
{
    __shared__ double red[32];
    const int b = blockIdx.x;
    double e = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int s = 0; s < nsplit; ++s) {
            const double2 v = as_c128(part[((size_t)s * P + p) * nb + b]);
            re += v.x;
            im += v.y;
        }
        e += lam[p] * (re * re + im * im);
    }
    e = block_sum(e, red);
    if (threadIdx.x == 0) out[b] = e;
}

// e[b] = kinetic + local (Parseval-normalised) + nonlocal
__global__ void combine_kernel(int nb, const double* __restrict__ kn, const double* __restrict__ loc,
                               const double* __restrict__ enl, double* __restrict__ e)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    double kin = 0.0, nrm = 0.0;
    for (int c = 0; c < KN_CHUNKS; ++c) {
        kin += kn[2 * (b * KN_CHUNKS + c)];
        nrm += kn[2 * (b * KN_CHUNKS + c) + 1];
    }
    const double s1 = loc[2 * b], s0 = loc[2 * b + 1];
    const double el = s0 > 0.0 ? s1 / s0 * nrm : 0.0;
    e[b] = kin + el + (enl ? enl[b] : 0.0);
}

// d[b] = Re sum_G conj(psi) h (the Rayleigh-quotient numerator)
__global__ void __launch_bounds__(256) dot_kernel(int npw, const double2* __restrict__ psi,
                                                  const double2* __restrict__ h, double* __restrict__ d)
{
    __shared__ double red[32];
    const size_t o = (size_t)blockIdx.x * npw;
    double s = 0.0;
    for (int g = threadIdx.x; g < npw; g += blockDim.x) s += psi[o + g].x * h[o + g].x + psi[o + g].y * h[o + g].y;
    s = block_sum(s, red);
    if (threadIdx.x == 0) d[blockIdx.x] = s;
}

__global__ void sub_kernel(int nb, const double* __restrict__ after, const double* __restrict__ before,
                           double* __restrict__ e)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) e[b] = after[b] - before[b];
}

// k·p sums of band n (one block per band of the lowest n_low):
//   S[n][a][b] = sum_{m != n, |E_n - E_m| > tol} Re(M_a[n][m] M_b[m][n]) / (E_n - E_m)
// with M_a[m][n] = <psi_m|dH/dk_a|psi_n> at M[(a nb + m) nb + n]; FP64.
__global__ void __launch_bounds__(256) kp_sums_kernel(int nb, const double2* __restrict__ M,
                                                      const double* __restrict__ E, double tol,
                                                      double* __restrict__ S, int* __restrict__ skipped)
{
    __shared__ double red[32];
    const int n = blockIdx.x;
    const size_t mm = (size_t)nb * nb;
    double acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = 0.0;
    double sk = 0.0;
    for (int m = threadIdx.x; m < nb; m += blockDim.x) {
        if (m == n) continue;
        const double de = E[n] - E[m];
        if (fabs(de) <= tol) {
            sk += 1.0;
            continue;
        }
        const double inv = 1.0 / de;
        double2 a[3], b[3];
#pragma unroll
        for (int al = 0; al < 3; ++al) {
            a[al] = M[al * mm + (size_t)n * nb + m];
            b[al] = M[al * mm + (size_t)m * nb + n];
        }
#pragma unroll
        for (int al = 0; al < 3; ++al)
#pragma unroll
            for (int be = 0; be < 3; ++be) acc[al * 3 + be] += (a[al].x * b[be].x - a[al].y * b[be].y) * inv;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double v = block_sum(acc[i], red);
        if (threadIdx.x == 0) S[(size_t)n * 9 + i] = v;
    }
    const double k = block_sum(sk, red);
    if (threadIdx.x == 0 && skipped) skipped[n] = (int)k;
}

}  // namespace

cudaError_t launch_kp_sums(int nb, int n_low, const double2* M, const double* E, double tol, double* S, int* skipped,
                           cudaStream_t st)
{
    if (n_low == 0) return cudaSuccess;
    kp_sums_kernel<<<n_low, 256, 0, st>>>(nb, M, E, tol, S, skipped);
    return cudaGetLastError();
}

cudaError_t launch_kin_norm(int npw, int nb, const double2* psi, const double* kinetic, double* out, cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    kin_norm_kernel<<<dim3(nb, KN_CHUNKS), 256, 0, st>>>(npw, psi, kinetic, out);
    return cudaGetLastError();
}

cudaError_t launch_local_sums(int nb, int nslots, const double* epart, double* out, cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    local_sums_kernel<<<nb, 256, 0, st>>>(nslots, epart, out);
    return cudaGetLastError();
}

template <typename Acc>
cudaError_t launch_nl_energy(int P, int nb, int nsplit, const Acc* part, const double* lam, double* out,
                             cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    nl_energy_kernel<Acc><<<nb, 256, 0, st>>>(P, nb, nsplit, part, lam, out);
    return cudaGetLastError();
}

cudaError_t launch_energy_combine(int nb, const double* kn, const double* loc, const double* enl, double* e,
                                  cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    combine_kernel<<<ceil_div(nb, 128), 128, 0, st>>>(nb, kn, loc, enl, e);
    return cudaGetLastError();
}

cudaError_t launch_band_dot(int npw, int nb, const double2* psi, const double2* h, double* d, cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    dot_kernel<<<nb, 256, 0, st>>>(npw, psi, h, d);
    return cudaGetLastError();
}

cudaError_t launch_band_sub(int nb, const double* after, const double* before, double* e, cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    sub_kernel<<<ceil_div(nb, 128), 128, 0, st>>>(nb, after, before, e);
    return cudaGetLastError();
}

template cudaError_t launch_nl_energy<double2>(int, int, int, const double2*, const double*, double*, cudaStream_t);
template cudaError_t launch_nl_energy<float2>(int, int, int, const float2*, const double*, double*, cudaStream_t);

int kin_norm_words(int nb) { return 2 * KN_CHUNKS * nb; }
