// selftest.cu — device check of the integer-pipe FP64 <-> FP32 conversions
// (d2f_bits, f2d_bits in common.cuh) against the hardware conversions.
#include <cuda_runtime.h>

#include "hpsi_gb300.h"
#include "common.cuh"
#include "tc_gemm.cuh"

namespace {

__global__ void convert_kernel(const double* __restrict__ x, long n, float* f_bits, float* f_hw, double* d_bits,
                               double* d_hw)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = __double2float_rn(v);
    f_bits[i] = d2f_bits(v);
    f_hw[i] = h;
    d_bits[i] = f2d_bits(h);
    d_hw[i] = (double)h;
}

}  // namespace

extern "C" int hpsi_selftest_convert(const double* x, long n, float* f_bits, float* f_hw, double* d_bits,
                                     double* d_hw)
{
    if (n < 0 || (n > 0 && (!x || !f_bits || !f_hw || !d_bits || !d_hw))) return HPSI_ERR_BAD_ARG;
    if (n == 0) return HPSI_OK;
    const size_t nd = (size_t)n * sizeof(double), nf = (size_t)n * sizeof(float);
    char* m = nullptr;
    if (cudaMalloc(&m, 3 * nd + 2 * nf) != cudaSuccess) return HPSI_ERR_OOM;
    double* dx = reinterpret_cast<double*>(m);
    double* db = dx + n;
    double* dh = db + n;
    float* fb = reinterpret_cast<float*>(dh + n);
    float* fh = fb + n;
    cudaError_t e = cudaMemcpy(dx, x, nd, cudaMemcpyHostToDevice);
    if (!e) {
        convert_kernel<<<ceil_div(n, 256), 256>>>(dx, n, fb, fh, db, dh);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(f_bits, fb, nf, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(f_hw, fh, nf, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(d_bits, db, nd, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(d_hw, dh, nd, cudaMemcpyDeviceToHost);
    cudaFree(m);
    return e ? HPSI_ERR_CUDA : HPSI_OK;
}

// Test hook of the bounded pipeline waits: lowers the poll limit of the
// tensor-core GEMMs' MMA issuer (0: it gives up at once) so that a test can
// watch a wait run out and the error reach the caller as HPSI_ERR_TIMEOUT.
extern "C" int hpsi_selftest_wait_limit(long polls)
{
    return tc_set_issue_wait_limit(polls) == cudaSuccess ? HPSI_OK : HPSI_ERR_CUDA;
}
