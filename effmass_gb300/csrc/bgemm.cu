// bgemm.cu — ragged batched SIMT complex GEMMs for the nonlocal term of many
// k-points at once (one launch for the projections of all k, one for the
// expansions).
//
// Reference: the per-projector passes of src/H_psi/hamiltonian_callable.cpp:259-297
//   inner = sum_G conj(p(G)) psi(G);   hpsi(G) += lambda * inner * p(G),
// written for item i (a k-point with its bands) as two GEMMs over the
// projector matrix Pr_i[P][npw_i]:
//   projection  part_i[s][P][nb_i] = conj(Pr_i) psi_i^T over the s-th K chunk
//   reduction   W_i[P][nb_i]       = lambda . sum_s part_i[s]  (sum in split order,
//                                   as in the unbatched path)
//   expansion   hpsi_i[nb_i][G]   += W_i^T Pr_i
//
// Tiles: a 16 x 16 thread grid owning TM x TN outputs each at stride 16, so
// the tile is (16 TM) x (16 TN) and shared-memory reads of a warp are
// conflict free.  The tile shape and the split count are chosen per batch by
// the autotuner of the batch plan.
#include <type_traits>
#include "kernels.cuh"

namespace {

template <typename Acc, typename T>
HPSI_D Acc bload(const T& v);
template <> HPSI_D double2 bload<double2, double2>(const double2& v) { return v; }
template <> HPSI_D float2 bload<float2, double2>(const double2& v) { return to_c64(v); }
template <> HPSI_D float2 bload<float2, float2>(const float2& v) { return v; }

constexpr int KS = 16;  // K slice staged per iteration

template <typename C, typename Acc, int TM, int TN>
__global__ void __launch_bounds__(256) bproj_kernel(int P, const BGemmItem* __restrict__ items, int nsplit,
                                                    Acc* __restrict__ part)
{
    using R = typename Real<Acc>::type;
    constexpr int BM = 16 * TM, BN = 16 * TN;
    __shared__ Acc As[KS][BM + 1];
    __shared__ Acc Bs[KS][BN + 1];
    const int it = blockIdx.z / nsplit, s = blockIdx.z - it * nsplit;
    const BGemmItem I = items[it];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (n0 >= I.nb) return;  // uniform: this item has fewer bands
    const C* A = static_cast<const C*>(I.pr);
    const int K = I.npw;
    const int kchunk = ((K + nsplit - 1) / nsplit + KS - 1) / KS * KS;
    const int kbeg = s * kchunk, kend = min(K, kbeg + kchunk);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R ar[TM][TN], ai[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) ar[i][j] = ai[i][j] = 0;
    for (int k0 = kbeg; k0 < kend; k0 += KS) {
        for (int e = threadIdx.x; e < BM * KS; e += 256) {
            const int r = e / KS, kk = e % KS, gk = k0 + kk;
            As[kk][r] = (m0 + r < P && gk < kend) ? bload<Acc>(A[(size_t)(m0 + r) * K + gk]) : cmake<Acc>(0, 0);
        }
        for (int e = threadIdx.x; e < BN * KS; e += 256) {
            const int r = e / KS, kk = e % KS, gk = k0 + kk;
            Bs[kk][r] = (n0 + r < I.nb && gk < kend) ? bload<Acc>(I.psi[(size_t)(n0 + r) * K + gk])
                                                     : cmake<Acc>(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KS; ++kk) {
            Acc a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    ar[i][j] += a[i].x * b[j].x + a[i].y * b[j].y;  // conj(a) * b
                    ai[i][j] += a[i].x * b[j].y - a[i].y * b[j].x;
                }
        }
        __syncthreads();
    }
    Acc* out = part + I.part_off + (size_t)s * P * I.nb;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= P) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n < I.nb) out[(size_t)m * I.nb + n] = cmake<Acc>(ar[i][j], ai[i][j]);
        }
    }
}

// W_i[m][n] = lam[m] * sum_s part_i[s][m][n] in split order (FP64 for
// complex128, compensated FP32 for complex64), one thread per (m, n);
// grid (ceil(P nb_max / 256), items).
template <typename C, typename Acc>
__global__ void __launch_bounds__(256) bred_kernel(int P, const BGemmItem* __restrict__ items, int nsplit,
                                                   const Acc* __restrict__ part, C* __restrict__ W)
{
    const BGemmItem I = items[blockIdx.y];
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= P * I.nb) return;
    const Acc* pw = part + I.part_off + idx;
    const size_t split_stride = (size_t)P * I.nb;
    if constexpr (std::is_same<Acc, float2>::value && std::is_same<C, float2>::value) {
        Sum2f re, im;  // complex64: compensated FP32, no FP64 pipe
        for (int s = 0; s < nsplit; ++s) {
            const float2 v = pw[s * split_stride];
            re.add(v.x);
            im.add(v.y);
        }
        const float l = d2f_bits(I.lam[idx / I.nb]);
        W[I.w_off + idx] = make_float2(l * re.value(), l * im.value());
        return;
    }
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < nsplit; ++s) {
        const double2 v = as_c128(pw[s * split_stride]);
        sr += v.x;
        si += v.y;
    }
    const double l = I.lam[idx / I.nb];
    W[I.w_off + idx] = from_c128<C>(make_double2(l * sr, l * si));
}

// hpsi_i[n][g] += sum_m W_i[m][n] Pr_i[m][g].  Block tile: (16 TM) bands x (16 TN) G.
template <typename C, int TM, int TN>
__global__ void __launch_bounds__(256) bexp_kernel(int P, const BGemmItem* __restrict__ items,
                                                   const C* __restrict__ W)
{
    using R = typename Real<C>::type;
    constexpr int BB = 16 * TM, BG = 16 * TN;
    __shared__ C Ws[KS][BB + 1];
    __shared__ C As[KS][BG + 1];
    const BGemmItem I = items[blockIdx.z];
    const int g0 = blockIdx.x * BG, n0 = blockIdx.y * BB;
    if (n0 >= I.nb || g0 >= I.npw) return;  // uniform
    const C* A = static_cast<const C*>(I.pr);
    const C* Wi = W + I.w_off;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    R ar[TM][TN], ai[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) ar[i][j] = ai[i][j] = 0;
    for (int m0 = 0; m0 < P; m0 += KS) {
        for (int e = threadIdx.x; e < KS * BB; e += 256) {
            const int mm = e / BB, c = e % BB, m = m0 + mm, n = n0 + c;
            Ws[mm][c] = (m < P && n < I.nb) ? Wi[(size_t)m * I.nb + n] : cmake<C>(0, 0);
        }
        for (int e = threadIdx.x; e < KS * BG; e += 256) {
            const int mm = e / BG, c = e % BG, m = m0 + mm, g = g0 + c;
            As[mm][c] = (m < P && g < I.npw) ? A[(size_t)m * I.npw + g] : cmake<C>(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int mm = 0; mm < KS; ++mm) {
            C w[TM], a[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) w[i] = Ws[mm][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) a[j] = As[mm][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    ar[i][j] += w[i].x * a[j].x - w[i].y * a[j].y;
                    ai[i][j] += w[i].x * a[j].y + w[i].y * a[j].x;
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
            const int n = n0 + ty + 16 * i, g = g0 + tx + 16 * j;
            o[i][j] = (n < I.nb && g < I.npw) ? I.hpsi[(size_t)n * I.npw + g] : make_double2(0.0, 0.0);
        }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + ty + 16 * i, g = g0 + tx + 16 * j;
            if (n < I.nb && g < I.npw) {
                o[i][j].x += (double)ar[i][j];
                o[i][j].y += (double)ai[i][j];
                I.hpsi[(size_t)n * I.npw + g] = o[i][j];
            }
        }
}

// (TM, TN) variants the tuner chooses from
constexpr int kTiles[][2] = {{1, 2}, {2, 2}, {1, 4}, {2, 4}, {4, 2}, {4, 4}};
constexpr int kNumTiles = sizeof(kTiles) / sizeof(kTiles[0]);

template <typename C, typename Acc, int T>
void proj_launch(dim3 g, int P, const BGemmItem* items, int nsplit, Acc* part, cudaStream_t st)
{
    bproj_kernel<C, Acc, kTiles[T][0], kTiles[T][1]><<<g, 256, 0, st>>>(P, items, nsplit, part);
}

template <typename C, int T>
void exp_launch(dim3 g, int P, const BGemmItem* items, const C* W, cudaStream_t st)
{
    bexp_kernel<C, kTiles[T][0], kTiles[T][1]><<<g, 256, 0, st>>>(P, items, W);
}

}  // namespace

int bgemm_tile_count() { return kNumTiles; }

void bgemm_tile_shape(int tile, int* tm, int* tn)
{
    *tm = kTiles[tile][0];
    *tn = kTiles[tile][1];
}

template <typename C, typename Acc>
cudaError_t launch_bproj(int P, const BGemmItem* items, int n_items, int nb_max, int nsplit, int tile, Acc* part,
                         cudaStream_t st)
{
    if (tile < 0 || tile >= kNumTiles || nsplit < 1) return cudaErrorInvalidValue;
    if (P == 0 || n_items == 0 || nb_max == 0) return cudaSuccess;
    dim3 g(ceil_div(P, 16 * kTiles[tile][0]), ceil_div(nb_max, 16 * kTiles[tile][1]), n_items * nsplit);
    switch (tile) {
        case 0: proj_launch<C, Acc, 0>(g, P, items, nsplit, part, st); break;
        case 1: proj_launch<C, Acc, 1>(g, P, items, nsplit, part, st); break;
        case 2: proj_launch<C, Acc, 2>(g, P, items, nsplit, part, st); break;
        case 3: proj_launch<C, Acc, 3>(g, P, items, nsplit, part, st); break;
        case 4: proj_launch<C, Acc, 4>(g, P, items, nsplit, part, st); break;
        default: proj_launch<C, Acc, 5>(g, P, items, nsplit, part, st); break;
    }
    return cudaGetLastError();
}

template <typename C, typename Acc>
cudaError_t launch_bexp(int P, const BGemmItem* items, int n_items, int nb_max, int npw_max, int nsplit, int tile,
                        const Acc* part, C* W, cudaStream_t st)
{
    if (tile < 0 || tile >= kNumTiles || nsplit < 1) return cudaErrorInvalidValue;
    if (P == 0 || n_items == 0 || nb_max == 0 || npw_max == 0) return cudaSuccess;
    bred_kernel<C, Acc><<<dim3(ceil_div((long)P * nb_max, 256), n_items), 256, 0, st>>>(P, items, nsplit, part, W);
    dim3 g(ceil_div(npw_max, 16 * kTiles[tile][1]), ceil_div(nb_max, 16 * kTiles[tile][0]), n_items);
    switch (tile) {
        case 0: exp_launch<C, 0>(g, P, items, W, st); break;
        case 1: exp_launch<C, 1>(g, P, items, W, st); break;
        case 2: exp_launch<C, 2>(g, P, items, W, st); break;
        case 3: exp_launch<C, 3>(g, P, items, W, st); break;
        case 4: exp_launch<C, 4>(g, P, items, W, st); break;
        default: exp_launch<C, 5>(g, P, items, W, st); break;
    }
    return cudaGetLastError();
}

template cudaError_t launch_bproj<double2, double2>(int, const BGemmItem*, int, int, int, int, double2*, cudaStream_t);
template cudaError_t launch_bproj<float2, float2>(int, const BGemmItem*, int, int, int, int, float2*, cudaStream_t);
template cudaError_t launch_bexp<double2, double2>(int, const BGemmItem*, int, int, int, int, int, const double2*,
                                                   double2*, cudaStream_t);
template cudaError_t launch_bexp<float2, float2>(int, const BGemmItem*, int, int, int, int, int, const float2*,
                                                 float2*, cudaStream_t);
