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
#include <type_traits>
#include "kernels.cuh"

template <typename Acc, typename T>
HPSI_D Acc load_as(const T& v);
template <> HPSI_D double2 load_as<double2, double2>(const double2& v) { return v; }
template <> HPSI_D float2 load_as<float2, double2>(const double2& v) { return to_c64(v); }
template <> HPSI_D float2 load_as<float2, float2>(const float2& v) { return v; }
template <> HPSI_D double2 load_as<double2, float2>(const float2& v) { return to_c128(v); }

constexpr int GB_K = 16;  // K slice staged per iteration

// Projection tile: (16 TM) x (16 TN) outputs per 256-thread block, each thread
// TM x TN at stride 16 (conflict-free shared-memory reads).  The launcher picks
// the tile from M and N so that small problems (a few bands, few projectors)
// do not spend the block on padding — FP64 runs at a small fraction of the
// FP32 rate on this part, so wasted FP64 work shows directly.
template <typename TA, typename TB, typename Acc, int TM, int TN>
__global__ void __launch_bounds__(256) proj_gemm_kernel(int M, int N, int K, const TA* __restrict__ A, size_t lda,
                                                        const TB* __restrict__ B, size_t ldb, Acc* __restrict__ part,
                                                        int kchunk)
{
    using R = typename Real<Acc>::type;
    constexpr int BM = 16 * TM, BN = 16 * TN;
    __shared__ Acc As[GB_K][BM + 1];
    __shared__ Acc Bs[GB_K][BN + 1];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, s = blockIdx.z;
    const int kbeg = s * kchunk;
    const int kend = min(K, kbeg + kchunk);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R accr[TM][TN], acci[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) accr[i][j] = acci[i][j] = 0;

    for (int k0 = kbeg; k0 < kend; k0 += GB_K) {
        for (int e = threadIdx.x; e < BM * GB_K; e += 256) {
            const int r = e / GB_K, kk = e % GB_K, gk = k0 + kk;
            As[kk][r] = (m0 + r < M && gk < kend) ? load_as<Acc>(A[(size_t)(m0 + r) * lda + gk]) : cmake<Acc>(0, 0);
        }
        for (int e = threadIdx.x; e < BN * GB_K; e += 256) {
            const int r = e / GB_K, kk = e % GB_K, gk = k0 + kk;
            Bs[kk][r] = (n0 + r < N && gk < kend) ? load_as<Acc>(B[(size_t)(n0 + r) * ldb + gk]) : cmake<Acc>(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            Acc a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    // conj(a) * b
                    accr[i][j] += a[i].x * b[j].x + a[i].y * b[j].y;
                    acci[i][j] += a[i].x * b[j].y - a[i].y * b[j].x;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n < N) part[((size_t)s * M + m) * N + n] = cmake<Acc>(accr[i][j], acci[i][j]);
        }
    }
}

static inline int tile_mult(int extent) { return extent <= 16 ? 1 : (extent <= 32 ? 2 : 4); }

template <typename TA, typename TB, typename Acc, int TM, int TN>
static void proj_launch(dim3 g, int M, int N, int K, const TA* A, size_t lda, const TB* B, size_t ldb, Acc* part,
                        int kchunk, cudaStream_t st)
{
    proj_gemm_kernel<TA, TB, Acc, TM, TN><<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, part, kchunk);
}

template <typename TA, typename TB, typename Acc>
cudaError_t launch_proj_gemm(int M, int N, int K, const TA* A, size_t lda, const TB* B, size_t ldb, Acc* part,
                             int nsplit, cudaStream_t st)
{
    if (M == 0 || N == 0) return cudaSuccess;
    int kchunk = ceil_div(K, nsplit);
    kchunk = ceil_div(kchunk, GB_K) * GB_K;
    const int tm = tile_mult(M), tn = tile_mult(N);
    dim3 g(ceil_div(M, 16 * tm), ceil_div(N, 16 * tn), nsplit);
    // nsplit partial slabs are written even when K is split finer than needed (empty chunks write zeros)
    if (tm == 1 && tn == 1) proj_launch<TA, TB, Acc, 1, 1>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tm == 1 && tn == 2) proj_launch<TA, TB, Acc, 1, 2>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tm == 2 && tn == 1) proj_launch<TA, TB, Acc, 2, 1>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tm == 2 && tn == 2) proj_launch<TA, TB, Acc, 2, 2>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tm == 1) proj_launch<TA, TB, Acc, 1, 4>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tn == 1) proj_launch<TA, TB, Acc, 4, 1>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tm == 2) proj_launch<TA, TB, Acc, 2, 4>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else if (tn == 2) proj_launch<TA, TB, Acc, 4, 2>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    else proj_launch<TA, TB, Acc, 4, 4>(g, M, N, K, A, lda, B, ldb, part, kchunk, st);
    return cudaGetLastError();
}

// Split count for a projection of an M x N result over K: enough blocks for
// every SM (two per SM), at least 64 of K per split.
int proj_gemm_splits(int M, int N, int K)
{
    const int blocks = ceil_div(M, 16 * tile_mult(M)) * ceil_div(N, 16 * tile_mult(N));
    const int want = ceil_div(2 * 152, blocks);
    const int maxs = K / 64 > 1 ? K / 64 : 1;
    return want < 1 ? 1 : (want < maxs ? want : maxs);
}

template <typename Acc, typename CW>
__global__ void reduce_splits_kernel(int M, int N, int nsplit, const Acc* __restrict__ part,
                                     const double* __restrict__ scale, int period, CW* __restrict__ W, size_t ldw)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)M * N) return;
    const int m = (int)(idx / N), n = (int)(idx % N);
    if constexpr (std::is_same<Acc, float2>::value && std::is_same<CW, float2>::value) {
        Sum2f re, im;  // complex64: compensated FP32, no FP64 pipe
        for (int s = 0; s < nsplit; ++s) {
            const float2 v = part[(size_t)s * M * N + idx];
            re.add(v.x);
            im.add(v.y);
        }
        const float f = scale ? d2f_bits(scale[m % period]) : 1.f;
        W[(size_t)m * ldw + n] = make_float2(f * re.value(), f * im.value());
        return;
    }
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

template <typename C, int TM, int TN>
__global__ void __launch_bounds__(256) expand_gemm_kernel(int M, int N, int K, const C* __restrict__ W, size_t ldw,
                                                          const C* __restrict__ A, size_t lda,
                                                          double2* __restrict__ out, size_t ldo)
{
    // out[n][k] += sum_m W[m][n] * A[m][k]; block tile: (16 TM) n x (16 TN) k, slices of 16 m
    using R = typename Real<C>::type;
    constexpr int BN = 16 * TM, BK = 16 * TN;
    __shared__ C Ws[GB_K][BN + 1];
    __shared__ C As[GB_K][BK + 1];
    const int k0 = blockIdx.x * BK, n0 = blockIdx.y * BN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R accr[TM][TN], acci[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) accr[i][j] = acci[i][j] = 0;
    for (int m0 = 0; m0 < M; m0 += GB_K) {
        for (int e = threadIdx.x; e < GB_K * BN; e += 256) {
            const int mm = e / BN, c = e % BN, gm = m0 + mm;
            Ws[mm][c] = (gm < M && n0 + c < N) ? W[(size_t)gm * ldw + n0 + c] : cmake<C>(0, 0);
        }
        for (int e = threadIdx.x; e < GB_K * BK; e += 256) {
            const int mm = e / BK, c = e % BK, gm = m0 + mm;
            As[mm][c] = (gm < M && k0 + c < K) ? A[(size_t)gm * lda + k0 + c] : cmake<C>(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int mm = 0; mm < GB_K; ++mm) {
            C w[TM], a[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) w[i] = Ws[mm][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) a[j] = As[mm][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    accr[i][j] += w[i].x * a[j].x - w[i].y * a[j].y;
                    acci[i][j] += w[i].x * a[j].y + w[i].y * a[j].x;
                }
        }
        __syncthreads();
    }
    // all loads of the read-modify-write first, so that they overlap
    double2 o[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + ty + 16 * i, k = k0 + tx + 16 * j;
            o[i][j] = (n < N && k < K) ? out[(size_t)n * ldo + k] : make_double2(0.0, 0.0);
        }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + ty + 16 * i, k = k0 + tx + 16 * j;
            if (n < N && k < K) {
                o[i][j].x += (double)accr[i][j];
                o[i][j].y += (double)acci[i][j];
                out[(size_t)n * ldo + k] = o[i][j];
            }
        }
}

template <typename C>
cudaError_t launch_expand_gemm(int M, int N, int K, const C* W, size_t ldw, const C* A, size_t lda, double2* out,
                               size_t ldo, cudaStream_t st)
{
    if (N == 0 || K == 0 || M == 0) return cudaSuccess;
    // few bands: a narrow band tile and four G-columns per thread
    if (N <= 16) {
        dim3 g(ceil_div(K, 64), ceil_div(N, 16));
        expand_gemm_kernel<C, 1, 4><<<g, 256, 0, st>>>(M, N, K, W, ldw, A, lda, out, ldo);
    } else if (N <= 32) {
        dim3 g(ceil_div(K, 64), ceil_div(N, 32));
        expand_gemm_kernel<C, 2, 4><<<g, 256, 0, st>>>(M, N, K, W, ldw, A, lda, out, ldo);
    } else {
        dim3 g(ceil_div(K, 64), ceil_div(N, 64));
        expand_gemm_kernel<C, 4, 4><<<g, 256, 0, st>>>(M, N, K, W, ldw, A, lda, out, ldo);
    }
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
