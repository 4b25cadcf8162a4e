// selftest_fft.cu — the device line transforms of the local term on a full
// grid, for known-answer tests (hpsi_selftest_fft3d).
//
// The reference's FFT3D (src/math/fft.cppm:60-85) transforms lines along z,
// then y, then x: G->r unnormalised with exp(+i..), r->G with exp(-i..) and
// 1/n per axis.  This entry point applies the same three axis passes with the
// transforms the H|psi> kernels are built from:
//   * complex128, and complex64 without a compile-time plan: the runtime-plan
//     Stockham stages of fft.cuh (fft_lines_io), one line per block in shared
//     memory;
//   * complex64 with a compile-time plan (n1 = n2 = n3 in {24, 36, 64, 72}):
//     the lane-pair transform of the plane kernels (fftreg::fft_pair) along z
//     and y, and the one-thread register transform of the x pass along x.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "hpsi_gb300.h"
#include "fft.cuh"
#include "fft_reg.cuh"

namespace {

// one line per block: element e of line L at g[base(L) + e * es], where the
// line's base walks the two other axes
template <typename C, bool WIDE>
__global__ void line_fft_kernel(C* g, int n, int es, int lines_inner, int stride_inner, int stride_outer, FftLen L,
                                FastDiv one, const C* __restrict__ tw_g, int sign, double scale)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* a = reinterpret_cast<C*>(smem_raw);
    C* b0 = a + n;
    C* b1 = b0 + n;
    C* tw = b1 + n;
    const int line = blockIdx.x;
    const size_t base = (size_t)(line % lines_inner) * stride_inner + (size_t)(line / lines_inner) * stride_outer;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        a[t] = g[base + (size_t)t * es];
        tw[t] = tw_g[t];
    }
    __syncthreads();
    const int r = fft_lines_io<C, true, WIDE>(SmemLines<C>{a, n, 1}, SmemLines<C>{a, n, 1}, b0, b1, L, one, n, 1, tw,
                                              sign);
    (void)r;
    __syncthreads();
    using R = typename Real<C>::type;
    for (int t = threadIdx.x; t < n; t += blockDim.x) g[base + (size_t)t * es] = cscale(a[t], (R)scale);
}

// lane-pair transform (the plane kernels' z / y transforms): lanes l and
// l ^ 16 share a line, the even lane holding the even samples; natural order
// out (each lane writes its half of the outputs)
template <typename PL, int S>
__global__ void line_fft_pair_kernel(float2* g, int es, int lines_inner, int stride_inner, int stride_outer,
                                     int nlines, float scale)
{
    constexpr int N = PL::n, H = N / 2, H1 = fftreg::PairPlan<N>::h1, H2 = fftreg::PairPlan<N>::h2;
    const int line = blockIdx.x * (blockDim.x / 2) + (threadIdx.x >> 5) * 16 + (threadIdx.x & 15);
    const bool odd = (threadIdx.x >> 4) & 1;
    const bool on = line < nlines;  // every lane runs the transform (full-warp exchange)
    float2* p = g + (on ? (size_t)(line % lines_inner) * stride_inner + (size_t)(line / lines_inner) * stride_outer : 0);
    float2 v[H];
#pragma unroll
    for (int n = 0; n < H; ++n) v[n] = on ? p[(size_t)(2 * n + (odd ? 1 : 0)) * es] : make_float2(0.f, 0.f);
    fftreg::fft_pair<S, H1, H2>(v, odd);
    if (on) {
#pragma unroll
        for (int m = 0; m < H; ++m) {
            const float2 e = v[fftreg::split_pos<H1, H2>(m)];
            p[(size_t)(m + (odd ? H : 0)) * es] = make_float2(e.x * scale, e.y * scale);
        }
    }
}

// register transform, one thread per line (the x pass's transform); natural
// order out (the split positions read back through split_pos)
template <typename PL, int S>
__global__ void line_fft_reg_kernel(float2* g, int es, int lines_inner, int stride_inner, int stride_outer, int nlines,
                                    float scale)
{
    constexpr int N1 = PL::r0, N2 = PL::r1, N = PL::n;
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    float2* p = g + (size_t)(line % lines_inner) * stride_inner + (size_t)(line / lines_inner) * stride_outer;
    float2 v[N];
#pragma unroll
    for (int x = 0; x < N; ++x) v[x] = p[(size_t)x * es];
    fftreg::fft_nat_to_split<S, N1, N2>(v);
#pragma unroll
    for (int x = 0; x < N; ++x) {
        const float2 e = v[fftreg::split_pos<N1, N2>(x)];
        p[(size_t)x * es] = make_float2(e.x * scale, e.y * scale);
    }
}

template <typename C>
std::vector<C> twiddles(int n)
{
    std::vector<C> t(n);
    for (int j = 0; j < n; ++j) {
        const double a = 2.0 * 3.14159265358979323846 * j / n;
        t[j] = cmake<C>((typename Real<C>::type)std::cos(a), (typename Real<C>::type)std::sin(a));
    }
    return t;
}

// (es, lines_inner, stride_inner, stride_outer) of the lines along axis d of an n1 x n2 x n3 grid
void axis_walk(int d, int n1, int n2, int n3, int* es, int* li, int* si, int* so)
{
    if (d == 2) { *es = 1; *li = n2; *si = n3; *so = n2 * n3; }          // z-lines: (i, j)
    else if (d == 1) { *es = n3; *li = n3; *si = 1; *so = n2 * n3; }    // y-lines: (i, k)
    else { *es = n2 * n3; *li = n2 * n3; *si = 1; *so = 0; }            // x-lines: (j, k)
}

template <typename C>
cudaError_t run_runtime_axis(C* d, int d_axis, int n1, int n2, int n3, int sign, cudaStream_t st)
{
    const int n[3] = {n1, n2, n3};
    FftLen L;
    if (!fft_factor(n[d_axis], &L)) return cudaErrorInvalidValue;
    std::vector<C> tw = twiddles<C>(n[d_axis]);
    C* dtw = nullptr;
    cudaError_t e = cudaMalloc(&dtw, tw.size() * sizeof(C));
    if (e) return e;
    cudaMemcpy(dtw, tw.data(), tw.size() * sizeof(C), cudaMemcpyHostToDevice);
    int es, li, si, so;
    axis_walk(d_axis, n1, n2, n3, &es, &li, &si, &so);
    const int nlines = n1 * n2 * n3 / n[d_axis];
    const double scale = sign < 0 ? 1.0 / n[d_axis] : 1.0;
    const size_t smem = 4 * sizeof(C) * (size_t)n[d_axis];
    if (fft_needs_wide(L)) {
        cudaFuncSetAttribute(line_fft_kernel<C, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        line_fft_kernel<C, true><<<nlines, 128, smem, st>>>(d, n[d_axis], es, li, si, so, L, make_fastdiv(1u), dtw, sign,
                                                             scale);
    } else {
        line_fft_kernel<C, false><<<nlines, 128, smem, st>>>(d, n[d_axis], es, li, si, so, L, make_fastdiv(1u), dtw,
                                                              sign, scale);
    }
    e = cudaGetLastError();
    cudaStreamSynchronize(st);
    cudaFree(dtw);
    return e;
}

template <typename PL>
cudaError_t run_plan_axes(float2* d, int sign, cudaStream_t st)
{
    constexpr int N = PL::n;
    const float scale = sign < 0 ? 1.0f / N : 1.0f;
    const int nlines = N * N;
    int es, li, si, so;
    for (int ax : {2, 1}) {  // z then y: lane-pair transforms, 64 lines per 128-thread block
        axis_walk(ax, N, N, N, &es, &li, &si, &so);
        if (sign > 0) line_fft_pair_kernel<PL, +1><<<(nlines + 63) / 64, 128, 0, st>>>(d, es, li, si, so, nlines, scale);
        else line_fft_pair_kernel<PL, -1><<<(nlines + 63) / 64, 128, 0, st>>>(d, es, li, si, so, nlines, scale);
    }
    axis_walk(0, N, N, N, &es, &li, &si, &so);  // x: one-thread register transform
    if (sign > 0) line_fft_reg_kernel<PL, +1><<<(nlines + 127) / 128, 128, 0, st>>>(d, es, li, si, so, nlines, scale);
    else line_fft_reg_kernel<PL, -1><<<(nlines + 127) / 128, 128, 0, st>>>(d, es, li, si, so, nlines, scale);
    const cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(st);
    return e;
}

}  // namespace

extern "C" int hpsi_selftest_fft3d(int n1, int n2, int n3, double* grid, int dir, int flags)
{
    if (n1 < 1 || n2 < 1 || n3 < 1 || !grid || (dir != 1 && dir != -1)) return HPSI_ERR_BAD_ARG;
    const int prec = flags & HPSI_PREC_MASK;
    if (prec != HPSI_PREC_FP64 && prec != HPSI_PREC_FP32) return HPSI_ERR_BAD_ARG;
    const int n[3] = {n1, n2, n3};
    for (int d = 0; d < 3; ++d) {
        FftLen L;
        if (!fft_factor(n[d], &L)) return HPSI_ERR_BAD_ARG;
    }
    const size_t total = (size_t)n1 * n2 * n3;
    cudaStream_t st = 0;
    cudaError_t e = cudaSuccess;
    if (prec == HPSI_PREC_FP64) {
        double2* d = nullptr;
        if ((e = cudaMalloc(&d, total * sizeof(double2)))) return HPSI_ERR_OOM;
        cudaMemcpy(d, grid, total * sizeof(double2), cudaMemcpyHostToDevice);
        for (int ax : {2, 1, 0})
            if (!e) e = run_runtime_axis<double2>(d, ax, n1, n2, n3, dir, st);
        if (!e) e = cudaMemcpy(grid, d, total * sizeof(double2), cudaMemcpyDeviceToHost);
        cudaFree(d);
        return e ? HPSI_ERR_CUDA : HPSI_OK;
    }
    std::vector<float2> h(total);
    for (size_t i = 0; i < total; ++i) h[i] = make_float2((float)grid[2 * i], (float)grid[2 * i + 1]);
    float2* d = nullptr;
    if ((e = cudaMalloc(&d, total * sizeof(float2)))) return HPSI_ERR_OOM;
    cudaMemcpy(d, h.data(), total * sizeof(float2), cudaMemcpyHostToDevice);
    FftLen L;
    fft_factor(n1, &L);
    const int id = fft_ct_id(L);
    if (n1 == n2 && n2 == n3 && id != FFT_CT_NONE) {
        switch (id) {
            case FFT_CT_72: e = run_plan_axes<FftPlan2<8, 9>>(d, dir, st); break;
            case FFT_CT_36: e = run_plan_axes<FftPlan2<9, 4>>(d, dir, st); break;
            case FFT_CT_24: e = run_plan_axes<FftPlan2<8, 3>>(d, dir, st); break;
            default: e = run_plan_axes<FftPlan2<8, 8>>(d, dir, st); break;
        }
    } else {
        for (int ax : {2, 1, 0})
            if (!e) e = run_runtime_axis<float2>(d, ax, n1, n2, n3, dir, st);
    }
    if (!e) e = cudaMemcpy(h.data(), d, total * sizeof(float2), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e) return HPSI_ERR_CUDA;
    for (size_t i = 0; i < total; ++i) {
        grid[2 * i] = h[i].x;
        grid[2 * i + 1] = h[i].y;
    }
    return HPSI_OK;
}
