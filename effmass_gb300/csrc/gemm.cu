// gemm.cu — register-tiled SIMT complex GEMMs for the nonlocal term
// (FP64 parity path and FP32 path).
//
// The reference applies each projector separately with two passes over the
// G-sphere per (atom, l, m, i) (src/H_psi/hamiltonian_callable.cpp:259-297):
//   inner = sum_G conj(p(G)) psi(G);   hpsi(G) += lambda * inner * p(G).
// For a block of nb bands these are two complex GEMMs over the projector
// matrix Pr[P][npw]:
//   projection  W[P][nb]   = conj(Pr) psi^T       (K = npw, split over K)
//   expansion   hpsi[nb][G] += (lambda W)^T Pr     (K = P)
// Tiles: 64 x 64 outputs per 256-thread block, 16-deep K slices staged in
// shared memory; each thread owns a 4 x 4 block of outputs at stride 16 so
// that shared-memory reads of a warp are bank-conflict free.
#include "kernels.cuh"

template <typename Acc, typename T>
HPSI_D Acc load_as(const T& v);
template <> HPSI_D double2 load_as<double2, double2>(const double2& v) { return v; }
template <> HPSI_D float2 load_as<float2, double2>(const double2& v) { return to_c64(v); }
template <> HPSI_D float2 load_as<float2, float2>(const float2& v) { return v; }
template <> HPSI_D double2 load_as<double2, float2>(const float2& v) { return to_c128(v); }

#define GB_M 64
#define GB_N 64
#define GB_K 16

template <typename TA, typename TB, typename Acc>
__global__ void __launch_bounds__(256) proj_gemm_kernel(int M, int N, int K, const TA* __restrict__ A, size_t lda,
                                                        const TB* __restrict__ B, size_t ldb, Acc* __restrict__ part,
                                                        int kchunk)
{
    using R = typename Real<Acc>::type;
    __shared__ Acc As[GB_K][GB_M + 1];
    __shared__ Acc Bs[GB_K][GB_N + 1];
    const int m0 = blockIdx.x * GB_M, n0 = blockIdx.y * GB_N, s = blockIdx.z;
    const int kbeg = s * kchunk;
    const int kend = min(K, kbeg + kchunk);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R accr[4][4], acci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) accr[i][j] = acci[i][j] = 0;

    for (int k0 = kbeg; k0 < kend; k0 += GB_K) {
        for (int e = threadIdx.x; e < GB_M * GB_K; e += 256) {
            const int r = e / GB_K, kk = e % GB_K;
            const int gm = m0 + r, gk = k0 + kk;
            Acc a = cmake<Acc>(0, 0), b = cmake<Acc>(0, 0);
            if (gm < M && gk < kend) a = load_as<Acc>(A[(size_t)gm * lda + gk]);
            if (n0 + r < N && gk < kend) b = load_as<Acc>(B[(size_t)(n0 + r) * ldb + gk]);
            As[kk][r] = a;
            Bs[kk][r] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            Acc a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // conj(a) * b
                    accr[i][j] += a[i].x * b[j].x + a[i].y * b[j].y;
                    acci[i][j] += a[i].x * b[j].y - a[i].y * b[j].x;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n < N) part[((size_t)s * M + m) * N + n] = cmake<Acc>(accr[i][j], acci[i][j]);
        }
    }
}

template <typename TA, typename TB, typename Acc>
cudaError_t launch_proj_gemm(int M, int N, int K, const TA* A, size_t lda, const TB* B, size_t ldb, Acc* part,
                             int nsplit, cudaStream_t st)
{
    if (M == 0 || N == 0) return cudaSuccess;
    int kchunk = ceil_div(K, nsplit);
    kchunk = ceil_div(kchunk, GB_K) * GB_K;
    dim3 g(ceil_div(M, GB_M), ceil_div(N, GB_N), nsplit);
    proj_gemm_kernel<TA, TB, Acc><<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, part, kchunk);
    return cudaGetLastError();
}

template <typename Acc, typename CW>
__global__ void reduce_splits_kernel(int M, int N, int nsplit, const Acc* __restrict__ part,
                                     const double* __restrict__ scale, int period, CW* __restrict__ W, size_t ldw)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)M * N) return;
    const int m = (int)(idx / N), n = (int)(idx % N);
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < nsplit; ++s) {
        double2 v = as_c128(part[(size_t)s * M * N + idx]);
        sr += v.x;
        si += v.y;
    }
    const double f = scale ? scale[m % period] : 1.0;
    W[(size_t)m * ldw + n] = from_c128<CW>(make_double2(f * sr, f * si));
}

template <typename Acc, typename CW>
cudaError_t launch_reduce_splits(int M, int N, int nsplit, const Acc* part, const double* scale, int scale_period,
                                 CW* W, size_t ldw, cudaStream_t st)
{
    size_t tot = (size_t)M * N;
    if (tot == 0) return cudaSuccess;
    reduce_splits_kernel<Acc, CW><<<ceil_div((long)tot, 256), 256, 0, st>>>(M, N, nsplit, part, scale,
                                                                           scale_period > 0 ? scale_period : M, W, ldw);
    return cudaGetLastError();
}

template <typename C>
__global__ void __launch_bounds__(256) expand_gemm_kernel(int M, int N, int K, const C* __restrict__ W, size_t ldw,
                                                          const C* __restrict__ A, size_t lda,
                                                          double2* __restrict__ out, size_t ldo)
{
    // out[n][k] += sum_m W[m][n] * A[m][k]; block tile: 64 n x 64 k, slices of 16 m
    using R = typename Real<C>::type;
    __shared__ C Ws[GB_K][GB_N + 1];
    __shared__ C As[GB_K][GB_M + 1];
    const int k0 = blockIdx.x * GB_M, n0 = blockIdx.y * GB_N;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R accr[4][4], acci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) accr[i][j] = acci[i][j] = 0;
    for (int m0 = 0; m0 < M; m0 += GB_K) {
        for (int e = threadIdx.x; e < GB_K * GB_M; e += 256) {
            const int mm = e / GB_M, c = e % GB_M;
            const int gm = m0 + mm;
            C w = cmake<C>(0, 0), a = cmake<C>(0, 0);
            if (gm < M && n0 + c < N) w = W[(size_t)gm * ldw + n0 + c];
            if (gm < M && k0 + c < K) a = A[(size_t)gm * lda + k0 + c];
            Ws[mm][c] = w;
            As[mm][c] = a;
        }
        __syncthreads();
#pragma unroll
        for (int mm = 0; mm < GB_K; ++mm) {
            C w[4], a[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] = Ws[mm][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) a[j] = As[mm][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    accr[i][j] += w[i].x * a[j].x - w[i].y * a[j].y;
                    acci[i][j] += w[i].x * a[j].y + w[i].y * a[j].x;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int n = n0 + ty + 16 * i;
        if (n >= N) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = k0 + tx + 16 * j;
            if (k < K) {
                double2 o = out[(size_t)n * ldo + k];
                o.x += (double)accr[i][j];
                o.y += (double)acci[i][j];
                out[(size_t)n * ldo + k] = o;
            }
        }
    }
}

template <typename C>
cudaError_t launch_expand_gemm(int M, int N, int K, const C* W, size_t ldw, const C* A, size_t lda, double2* out,
                               size_t ldo, cudaStream_t st)
{
    if (N == 0 || K == 0 || M == 0) return cudaSuccess;
    dim3 g(ceil_div(K, GB_M), ceil_div(N, GB_N));
    expand_gemm_kernel<C><<<g, 256, 0, st>>>(M, N, K, W, ldw, A, lda, out, ldo);
    return cudaGetLastError();
}

template <typename C>
__global__ void convert_kernel(size_t n, const double2* __restrict__ in, C* __restrict__ out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = from_c128<C>(in[i]);
}

template <typename C>
cudaError_t launch_convert(size_t n, const double2* in, C* out, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    convert_kernel<C><<<ceil_div((long)n, 256), 256, 0, st>>>(n, in, out);
    return cudaGetLastError();
}

// instantiations
template cudaError_t launch_proj_gemm<double2, double2, double2>(int, int, int, const double2*, size_t, const double2*,
                                                                 size_t, double2*, int, cudaStream_t);
template cudaError_t launch_proj_gemm<float2, float2, float2>(int, int, int, const float2*, size_t, const float2*,
                                                              size_t, float2*, int, cudaStream_t);
template cudaError_t launch_proj_gemm<float2, double2, float2>(int, int, int, const float2*, size_t, const double2*,
                                                               size_t, float2*, int, cudaStream_t);
template cudaError_t launch_proj_gemm<double2, double2, float2>(int, int, int, const double2*, size_t, const double2*,
                                                                size_t, float2*, int, cudaStream_t);
template cudaError_t launch_reduce_splits<double2, double2>(int, int, int, const double2*, const double*, int,
                                                            double2*, size_t, cudaStream_t);
template cudaError_t launch_reduce_splits<float2, float2>(int, int, int, const float2*, const double*, int, float2*,
                                                          size_t, cudaStream_t);
template cudaError_t launch_reduce_splits<float2, double2>(int, int, int, const float2*, const double*, int, double2*,
                                                           size_t, cudaStream_t);
template cudaError_t launch_reduce_splits<double2, float2>(int, int, int, const double2*, const double*, int, float2*,
                                                           size_t, cudaStream_t);
template cudaError_t launch_expand_gemm<double2>(int, int, int, const double2*, size_t, const double2*, size_t,
                                                 double2*, size_t, cudaStream_t);
template cudaError_t launch_expand_gemm<float2>(int, int, int, const float2*, size_t, const float2*, size_t, double2*,
                                                size_t, cudaStream_t);
template cudaError_t launch_convert<float2>(size_t, const double2*, float2*, cudaStream_t);
