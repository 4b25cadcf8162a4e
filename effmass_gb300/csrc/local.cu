// local.cu — kinetic + local-potential term of H|psi>, batched over bands.
//
// Reference: src/H_psi/hamiltonian_callable.cpp:119-182 — kinetic loop,
// scatter of psi(G) onto the grid at (g mod n), FFT3D G2R (unnormalised,
// exp(+iG.r)), multiply by V(r), FFT3D R2G (forward, 1/n per axis), gather.
//
// GB300 layout: the sphere occupies only nxs of the n1 x-planes, so the work
// is split into three passes over an intermediate T[band][plane][j][k]
// (complex, nxs planes of n2*n3):
//   A  g2r_planes : per (plane, band): scatter psi into a shared-memory plane,
//                   FFT along z then y (G2R), store the plane to T.
//   B  x_pass     : per (j, k-tile), looping over bands: gather the nxs
//                   planes of T into shared memory x-lines (zeros elsewhere),
//                   FFT along x (G2R), multiply by V, FFT along x (R2G), and
//                   store the nxs sphere planes back into T in place.
//   C  r2g_planes : per (plane, band): FFT along y then z (R2G), then gather
//                   the sphere points: hpsi += kinetic*psi + grid/N.
// T is sized for a chunk of bands so that it stays resident in L2 between
// the passes.  Kinetic energy is fused into pass C.
#include "fft.cuh"
#include "kernels.cuh"

// Launch shape per precision: complex64 kernels run 512-thread plane blocks
// (two per SM) and four x-pass blocks per SM; complex128 kernels keep the
// register budget of one block per SM.
template <typename C> struct Cfg;
template <> struct Cfg<float2> { static constexpr int plane_threads = 512, plane_min = 2, x_min = 4; };
template <> struct Cfg<double2> { static constexpr int plane_threads = 256, plane_min = 1, x_min = 1; };

// Shared-memory planes use a padded row stride n3p = n3 + 1 (odd) so that
// both the z-lines (rows) and the y-lines (columns) are read and written by
// consecutive threads without bank conflicts (both transforms walk lines
// fastest: LINE_FAST).
template <typename C, bool WIDE>
__global__ void __launch_bounds__(Cfg<C>::plane_threads, Cfg<C>::plane_min) g2r_planes(LocalArgs a, const double2* __restrict__ psi, C* __restrict__ T,
                                                  const C* __restrict__ tw_y_g, const C* __restrict__ tw_z_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n2 = a.n2, n3 = a.n3, n3p = n3 + 1, n23 = n2 * n3, n23p = n2 * n3p;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n23p;
    C* twy = b1 + n23p;
    C* twz = twy + n2;
    const int p = blockIdx.x;
    const int b = blockIdx.y;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) twy[t] = tw_y_g[t];
    for (int t = threadIdx.x; t < n3; t += blockDim.x) twz[t] = tw_z_g[t];
    for (int t = threadIdx.x; t < n23p; t += blockDim.x) b0[t] = cmake<C>(0, 0);
    __syncthreads();
    const double2* ps = psi + (size_t)b * a.npw;
    const int e0 = a.plane_off[p], e1 = a.plane_off[p + 1];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int ig = a.ent_ig[e];
        if (ig >= 0) {
            int jk = a.ent_jk[e];
            int j = jk / n3, k = jk - j * n3;
            b0[j * n3p + k] = from_c128<C>(ps[ig]);
        }
    }
    __syncthreads();
    int cur = fft_lines<C, true, WIDE>(b0, b1, 0, a.Lz, a.nl_z, n3p, 1, twz, +1);
    cur = fft_lines<C, true, WIDE>(b0, b1, cur, a.Ly, a.nl_y, 1, n3p, twy, +1);
    const C* res = cur ? b1 : b0;
    C* out = T + ((size_t)b * a.nxs + p) * n23;
    for (int t = threadIdx.x; t < n23; t += blockDim.x) {
        int j = t / n3, k = t - j * n3;
        out[t] = res[j * n3p + k];
    }
}

// x pass: a block owns the x-lines of (j, k0..k0+KT) for BB consecutive bands
// (NL = KT*BB lines, line L = bb*KT + kk, element x at [x*NL + L]); the V tile
// is loaded once per block.
template <typename C, typename V, bool WIDE>
__global__ void __launch_bounds__(256, Cfg<C>::x_min) x_pass(LocalArgs a, int nb, C* __restrict__ T, const V* __restrict__ vloc,
                                              const C* __restrict__ tw_x_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3, KT = a.kt, BB = a.bb, NL = KT * BB;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n1 * NL;
    C* twx = b1 + n1 * NL;
    V* vt = reinterpret_cast<V*>(twx + n1);
    const int j = blockIdx.y;
    const int k0 = blockIdx.x * KT;
    const int kt = min(KT, n3 - k0);
    const int bb0 = blockIdx.z * BB;
    const int nbb = min(BB, nb - bb0);
    const int nxs = a.nxs;
    const size_t plane = (size_t)n2 * n3;
    for (int t = threadIdx.x; t < n1; t += blockDim.x) twx[t] = tw_x_g[t];
    for (int t = threadIdx.x; t < n1 * kt; t += blockDim.x) {
        int x = t / kt, kk = t % kt;
        vt[x * KT + kk] = vloc[((size_t)x * n2 + j) * n3 + k0 + kk];
    }
    for (int t = threadIdx.x; t < n1 * NL; t += blockDim.x) b0[t] = cmake<C>(0, 0);
    __syncthreads();
    const int per_plane = nbb * kt;
    for (int t = threadIdx.x; t < nxs * per_plane; t += blockDim.x) {
        int pp = t / per_plane, r = t - pp * per_plane;
        int bb = r / kt, kk = r - bb * kt;
        const C* src = T + ((size_t)(bb0 + bb) * nxs + pp) * plane + (size_t)j * n3 + k0 + kk;
        b0[a.plane_x[pp] * NL + bb * KT + kk] = *src;
    }
    __syncthreads();
    int cur = fft_lines<C, true, WIDE>(b0, b1, 0, a.Lx, a.nl_x, 1, NL, twx, +1);
    C* res = cur ? b1 : b0;
    for (int t = threadIdx.x; t < n1 * NL; t += blockDim.x) {
        int x = t / NL, L = t - x * NL;
        int kk = L % KT;
        res[t] = cscale(res[t], (typename Real<C>::type)vt[x * KT + kk]);
    }
    __syncthreads();
    cur = fft_lines<C, true, WIDE>(b0, b1, cur, a.Lx, a.nl_x, 1, NL, twx, -1);
    res = cur ? b1 : b0;
    for (int t = threadIdx.x; t < nxs * per_plane; t += blockDim.x) {
        int pp = t / per_plane, r = t - pp * per_plane;
        int bb = r / kt, kk = r - bb * kt;
        C* dst = T + ((size_t)(bb0 + bb) * nxs + pp) * plane + (size_t)j * n3 + k0 + kk;
        *dst = res[a.plane_x[pp] * NL + bb * KT + kk];
    }
}

template <typename C, bool WIDE>
__global__ void __launch_bounds__(Cfg<C>::plane_threads, Cfg<C>::plane_min) r2g_planes(LocalArgs a, const C* __restrict__ T, const double2* __restrict__ psi,
                                                  double2* __restrict__ hpsi, const double* __restrict__ kinetic,
                                                  const C* __restrict__ tw_y_g, const C* __restrict__ tw_z_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n2 = a.n2, n3 = a.n3, n3p = n3 + 1, n23 = n2 * n3, n23p = n2 * n3p;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n23p;
    C* twy = b1 + n23p;
    C* twz = twy + n2;
    const int p = blockIdx.x;
    const int b = blockIdx.y;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) twy[t] = tw_y_g[t];
    for (int t = threadIdx.x; t < n3; t += blockDim.x) twz[t] = tw_z_g[t];
    const C* in = T + ((size_t)b * a.nxs + p) * n23;
    for (int t = threadIdx.x; t < n23; t += blockDim.x) {
        int j = t / n3, k = t - j * n3;
        b0[j * n3p + k] = in[t];
    }
    __syncthreads();
    int cur = fft_lines<C, true, WIDE>(b0, b1, 0, a.Ly, a.nl_y, 1, n3p, twy, -1);
    cur = fft_lines<C, true, WIDE>(b0, b1, cur, a.Lz, a.nl_z, n3p, 1, twz, -1);
    const C* res = cur ? b1 : b0;
    const double2* ps = psi + (size_t)b * a.npw;
    double2* hp = hpsi + (size_t)b * a.npw;
    const int e0 = a.plane_off[p], e1 = a.plane_off[p + 1];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int ig = a.ent_ig[e] & 0x7fffffff;
        int jk = a.ent_jk[e];
        int j = jk / n3, k = jk - j * n3;
        double2 g = as_c128(res[j * n3p + k]);
        double2 s = ps[ig];
        double kin = kinetic[ig];
        double2 h = hp[ig];
        h.x += kin * s.x + g.x * a.inv_n;
        h.y += kin * s.y + g.y * a.inv_n;
        hp[ig] = h;
    }
}

template <typename C>
static size_t plane_smem(const LocalArgs& a)
{
    return sizeof(C) * (2 * (size_t)a.n2 * (a.n3 + 1) + a.n2 + a.n3);
}

template <typename C, typename V>
static size_t xpass_smem(const LocalArgs& a)
{
    const size_t NL = (size_t)a.kt * a.bb;
    return sizeof(C) * (2 * (size_t)a.n1 * NL + a.n1) + sizeof(V) * (size_t)a.n1 * a.kt;
}

size_t local_smem_bytes(const LocalArgs& a, bool fp64)
{
    LocalArgs b = a;
    local_xpass_shape(&b, fp64 ? sizeof(double2) : sizeof(float2));
    size_t p = fp64 ? plane_smem<double2>(b) : plane_smem<float2>(b);
    size_t x = fp64 ? xpass_smem<double2, double>(b) : xpass_smem<float2, float>(b);
    return p > x ? p : x;
}

// x-pass block shape: about 48 KB of complex64 line buffers (four blocks per
// SM) or 96 KB of complex128 ones, at most 8 z-values per block, the rest
// filled with bands.
void local_xpass_shape(LocalArgs* a, size_t csize)
{
    const size_t budget = csize == 8 ? 48 * 1024 : 96 * 1024;
    int nlmax = (int)(budget / (2 * (size_t)a->n1 * csize));
    if (nlmax < 1) nlmax = 1;
    a->kt = nlmax < 8 ? nlmax : 8;
    if (a->kt > a->n3) a->kt = a->n3;
    a->bb = nlmax / a->kt;
    if (a->bb < 1) a->bb = 1;
    a->nl_z = make_fastdiv((uint32_t)a->n2);
    a->nl_y = make_fastdiv((uint32_t)a->n3);
    a->nl_x = make_fastdiv((uint32_t)(a->kt * a->bb));
}

template <typename C, typename V, bool WIDE>
static cudaError_t launch_local_t(const LocalArgs& a, int nb, const double2* psi, double2* hpsi, const double* kinetic,
                                  C* T, const V* vloc, const C* twx, const C* twy, const C* twz, cudaStream_t st,
                                  Prof* prof)
{
    const size_t sp = plane_smem<C>(a), sx = xpass_smem<C, V>(a);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(g2r_planes<C, WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(r2g_planes<C, WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(x_pass<C, V, WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx)))
        return e;
    if (a.nxs == 0 || nb == 0) return cudaSuccess;
    dim3 gp(a.nxs, nb);
    int h = prof->open(PH_G2R, st);
    g2r_planes<C, WIDE><<<gp, Cfg<C>::plane_threads, sp, st>>>(a, psi, T, twy, twz);
    prof->close(h, st);
    dim3 gx(ceil_div(a.n3, a.kt), a.n2, ceil_div(nb, a.bb));
    h = prof->open(PH_XPASS, st);
    x_pass<C, V, WIDE><<<gx, 256, sx, st>>>(a, nb, T, vloc, twx);
    prof->close(h, st);
    h = prof->open(PH_R2G, st);
    r2g_planes<C, WIDE><<<gp, Cfg<C>::plane_threads, sp, st>>>(a, T, psi, hpsi, kinetic, twy, twz);
    prof->close(h, st);
    return cudaGetLastError();
}

template <typename C, typename V>
cudaError_t launch_local(const LocalArgs& a, int nb, const double2* psi, double2* hpsi, const double* kinetic, C* T,
                         const V* vloc, const C* twx, const C* twy, const C* twz, cudaStream_t st, Prof* prof)
{
    const bool wide = fft_needs_wide(a.Lx) || fft_needs_wide(a.Ly) || fft_needs_wide(a.Lz);
    if (wide) return launch_local_t<C, V, true>(a, nb, psi, hpsi, kinetic, T, vloc, twx, twy, twz, st, prof);
    return launch_local_t<C, V, false>(a, nb, psi, hpsi, kinetic, T, vloc, twx, twy, twz, st, prof);
}

template cudaError_t launch_local<double2, double>(const LocalArgs&, int, const double2*, double2*, const double*,
                                                   double2*, const double*, const double2*, const double2*,
                                                   const double2*, cudaStream_t, Prof*);
template cudaError_t launch_local<float2, float>(const LocalArgs&, int, const double2*, double2*, const double*,
                                                 float2*, const float*, const float2*, const float2*, const float2*,
                                                 cudaStream_t, Prof*);
