// sternheimer.cu — FP64 vector kernels of the batched preconditioned CG that
// solves the Sternheimer equations for dpsi/dk (hpsi_sternheimer).
//
// For each occupied band n (all bands at once, one CG per band):
//   A_n x_n = b_n,   A_n = P_c (H - e_n) P_c + s P_v,   b_n = -P_c dH/dk_a psi_n
// with P_v = sum_m |psi_m><psi_m| over the occupied bands and P_c = 1 - P_v.
// The kernels here are the band-batched BLAS-1 pieces (one block per band for
// the reductions, in a fixed order) and the diagonal preconditioner; the
// occupied-space projections use the SIMT GEMMs, H the chosen H|psi> path.
#include "kernels.cuh"

namespace {

__device__ __forceinline__ double block_sum_d(double v, double* red)
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
    return r;
}

// d[b] = Re <x_b|y_b>   (one block per band)
__global__ void __launch_bounds__(256) bdot_kernel(int n, const double2* __restrict__ x, const double2* __restrict__ y,
                                                   double* __restrict__ d)
{
    __shared__ double red[32];
    const size_t o = (size_t)blockIdx.x * n;
    double s = 0.0;
    for (int g = threadIdx.x; g < n; g += blockDim.x) s += x[o + g].x * y[o + g].x + x[o + g].y * y[o + g].y;
    s = block_sum_d(s, red);
    if (threadIdx.x == 0) d[blockIdx.x] = s;
}

// y_b = alpha_b x_b + beta_b y_b  (alpha/beta per band; null alpha = 1, null beta = 0 ... see flags)
__global__ void baxpby_kernel(int n, int nb, const double* __restrict__ alpha, const double2* __restrict__ x,
                              const double* __restrict__ beta, double2* __restrict__ y, double asign, int mode)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * nb) return;
    const int b = (int)(i / n);
    const double a = asign * (alpha ? alpha[b] : 1.0);
    const double2 xv = x[i];
    double2 yv = y[i];
    if (mode == 0) {          // y += a x
        yv.x += a * xv.x;
        yv.y += a * xv.y;
    } else {                  // y = a x + beta y   (beta per band)
        const double bt = beta[b];
        yv.x = a * xv.x + bt * yv.x;
        yv.y = a * xv.y + bt * yv.y;
    }
    y[i] = yv;
}

// y_b += c_b * x_b with c_b = scale * e[b] (the -e_n x_n term of A_n)
__global__ void bscale_add_kernel(int n, int nb, const double* __restrict__ e, double scale,
                                  const double2* __restrict__ x, double2* __restrict__ y)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * nb) return;
    const double c = scale * e[i / n];
    y[i].x += c * x[i].x;
    y[i].y += c * x[i].y;
}

// z = M^-1 r with M_b(G) = max(kinetic(G) - e_b, 0) + tau (a positive diagonal)
__global__ void bprec_kernel(int n, int nb, const double* __restrict__ kin, const double* __restrict__ e, double tau,
                             const double2* __restrict__ r, double2* __restrict__ z)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * nb) return;
    const int b = (int)(i / n), g = (int)(i - (size_t)b * n);
    const double m = fmax(kin[g] - e[b], 0.0) + tau;
    z[i].x = r[i].x / m;
    z[i].y = r[i].y / m;
}

// ratio[b] = active ? num[b] / den[b] : 0 (den > 0); the per-band CG scalars
__global__ void bratio_kernel(int nb, const double* __restrict__ num, const double* __restrict__ den,
                              const int* __restrict__ active, double* __restrict__ out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    out[b] = (active[b] && den[b] > 0.0) ? num[b] / den[b] : 0.0;
}

}  // namespace

cudaError_t launch_bdot(int n, int nb, const double2* x, const double2* y, double* d, cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    bdot_kernel<<<nb, 256, 0, st>>>(n, x, y, d);
    return cudaGetLastError();
}

cudaError_t launch_baxpy(int n, int nb, const double* alpha, double asign, const double2* x, double2* y,
                         cudaStream_t st)
{
    const size_t tot = (size_t)n * nb;
    if (tot == 0) return cudaSuccess;
    baxpby_kernel<<<ceil_div((long)tot, 256), 256, 0, st>>>(n, nb, alpha, x, nullptr, y, asign, 0);
    return cudaGetLastError();
}

cudaError_t launch_baxpby(int n, int nb, const double* alpha, double asign, const double2* x, const double* beta,
                          double2* y, cudaStream_t st)
{
    const size_t tot = (size_t)n * nb;
    if (tot == 0) return cudaSuccess;
    baxpby_kernel<<<ceil_div((long)tot, 256), 256, 0, st>>>(n, nb, alpha, x, beta, y, asign, 1);
    return cudaGetLastError();
}

cudaError_t launch_bscale_add(int n, int nb, const double* e, double scale, const double2* x, double2* y,
                              cudaStream_t st)
{
    const size_t tot = (size_t)n * nb;
    if (tot == 0) return cudaSuccess;
    bscale_add_kernel<<<ceil_div((long)tot, 256), 256, 0, st>>>(n, nb, e, scale, x, y);
    return cudaGetLastError();
}

cudaError_t launch_bprec(int n, int nb, const double* kin, const double* e, double tau, const double2* r, double2* z,
                         cudaStream_t st)
{
    const size_t tot = (size_t)n * nb;
    if (tot == 0) return cudaSuccess;
    bprec_kernel<<<ceil_div((long)tot, 256), 256, 0, st>>>(n, nb, kin, e, tau, r, z);
    return cudaGetLastError();
}

cudaError_t launch_bratio(int nb, const double* num, const double* den, const int* active, double* out,
                          cudaStream_t st)
{
    if (nb == 0) return cudaSuccess;
    bratio_kernel<<<ceil_div(nb, 128), 128, 0, st>>>(nb, num, den, active, out);
    return cudaGetLastError();
}
