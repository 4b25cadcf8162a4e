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
// T holds a chunk of bands of at most 512 MB: wide launches fill the 152 SMs
// for every pass, which measured faster than chunks small enough to stay in
// L2 between the passes.  Kinetic energy is fused into pass C.
#include <type_traits>

#include "fft.cuh"
#include "fft_reg.cuh"
#include "kernels.cuh"

// Launch shape per precision: complex64 kernels run two 768-thread plane
// blocks per SM and four or five x-pass blocks per SM;
// complex128 kernels keep the register budget of one block per SM.
template <typename C> struct Cfg;
template <> struct Cfg<float2> {
    // 768-thread plane blocks, two per SM (48 warps): g2r_planes fits 40
    // registers without spills; r2g_planes spills 44 bytes there and still
    // measured faster than at 512 threads (0.139 vs 0.141 ms, 64-atom cell)
    static constexpr int plane_threads = 768, g2r_threads = 768, plane_min = 2, x_min = 4;
};
template <> struct Cfg<double2> {
    static constexpr int plane_threads = 256, g2r_threads = 256, plane_min = 1, x_min = 1;
};

// Plan tag of the kernels that run the runtime FFT plans
struct NoPlan {};

// Resident x-pass blocks per SM (the launch-bounds minimum): the complex64
// compile-time plans fit 48 registers without spills, so five 256-thread
// blocks (62.5% of the warp slots; ~39 KB of shared memory each) share an
// SM; the runtime-plan and wide-radix kernels keep their larger budgets.
template <typename C, bool WIDE, typename PL>
constexpr int xpass_min()
{
    if constexpr (WIDE) return (Cfg<C>::x_min + 1) / 2;
    else if constexpr (std::is_same<C, float2>::value && !std::is_same<PL, NoPlan>::value) return 5;
    else return Cfg<C>::x_min;
}

// Transform of a kernel's lines: the runtime plan (NoPlan) or a compile-time
// two-stage plan (FftPlan2) chosen by the host for common grid lengths.
template <typename C, bool WIDE, typename PL, typename LD, typename ST>
HPSI_D void lines(const LD& ld, const ST& st, C* bufA, C* bufB, const FftLen& L, const FastDiv& nlf, int ls, int es,
                  const C* tw, int sign)
{
    if constexpr (std::is_same<PL, NoPlan>::value) fft_lines_io<C, true, WIDE>(ld, st, bufA, bufB, L, nlf, ls, es, tw, sign);
    else fft_lines_ct<C, PL>(ld, st, bufA, nlf, ls, es, tw, sign);
}

// Shared-memory planes use a padded row stride n3p = n3 + 1 (odd) so that
// both the z-lines (rows) and the y-lines (columns) are read and written by
// consecutive threads without bank conflicts (both transforms walk lines
// fastest: LINE_FAST).  The first stage of a transform reads its source
// directly and the last stage writes its destination directly
// (fft_lines_io), so a plane costs two barriers per axis.

// global plane of T as y-lines: line = k, element = j
template <typename C>
struct PlaneGlobal {
    C* p;
    int n3;
    HPSI_D C operator()(int L, int e) const { return p[e * n3 + L]; }
    HPSI_D void operator()(int L, int e, C v) const { p[e * n3 + L] = v; }
};

// global plane of T as y-lines with a compile-time row length N3
template <typename C, int N3>
struct PlaneGlobalC {
    C* p;
    HPSI_D C operator()(int L, int e) const { return p[e * N3 + L]; }
    HPSI_D void operator()(int L, int e, C v) const { p[e * N3 + L] = v; }
};

// grid length of an axis: the compile-time plan's when there is one (then all
// three axes share it), else the runtime value
template <typename PL>
HPSI_D int plan_n(int runtime)
{
    if constexpr (std::is_same<PL, NoPlan>::value) return runtime;
    else return PL::n;
}

template <typename C, bool WIDE, typename PL>
__global__ void __launch_bounds__(Cfg<C>::g2r_threads, WIDE ? 1 : Cfg<C>::plane_min) g2r_planes(LocalArgs a, const double2* __restrict__ psi, C* __restrict__ T,
                                                  const C* __restrict__ tw_y_g, const C* __restrict__ tw_z_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n2 = plan_n<PL>(a.n2), n3 = plan_n<PL>(a.n3), n3p = n3 + 1, n23 = n2 * n3, n23p = n2 * n3p;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n23p;
    C* twy = b1 + n23p;
    C* twz = twy + n2;
    const int p = blockIdx.x;
    int b = blockIdx.y;
    int npw = a.npw, nxs = a.nxs;
    const int *plane_off = a.plane_off, *ent_ig = a.ent_ig, *ent_jk = a.ent_jk, *plane_jr = a.plane_jr;
    if (a.items) {  // batched: the band's item (uniform per block, before any barrier)
        const LocalItem I = a.items[a.band_item[b]];
        if (p >= I.nxs) return;
        b -= I.band0;
        npw = I.npw; nxs = I.nxs;
        plane_off = I.plane_off; ent_ig = I.ent_ig; ent_jk = I.ent_jk; plane_jr = I.plane_jr;
        psi = I.psi;
        T += I.t_off;
    }
    for (int t = threadIdx.x; t < n2; t += blockDim.x) twy[t] = tw_y_g[t];
    for (int t = threadIdx.x; t < n3; t += blockDim.x) twz[t] = tw_z_g[t];
    for (int t = threadIdx.x; t < n23p; t += blockDim.x) b0[t] = cmake<C>(0, 0);
    __syncthreads();
    const double2* ps = psi + (size_t)b * npw;
    const int e0 = plane_off[p], e1 = plane_off[p + 1];
    uint32_t mx = 0u;  // float bits of the largest |re|, |im| this thread scattered
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int ig = ent_ig[e];
        if (ig >= 0) {
            int jk = ent_jk[e];
            int j = jk / n3, k = jk - j * n3;
            const C v = from_c128<C>(ps[ig]);
            b0[j * n3p + k] = v;
            if constexpr (std::is_same<C, float2>::value)
                mx = max(mx, max(__float_as_uint(v.x) & 0x7fffffffu, __float_as_uint(v.y) & 0x7fffffffu));
        } else if constexpr (std::is_same<C, float2>::value) {
            // a G that shares its grid point with a later one: not scattered,
            // but its coefficient is still a row element of the band operand
            if (a.rowmax && !a.items) {
                const float2 v = to_c64(ps[ig & 0x7fffffff]);
                mx = max(mx, max(__float_as_uint(v.x) & 0x7fffffffu, __float_as_uint(v.y) & 0x7fffffffu));
            }
        }
    }
    if constexpr (std::is_same<C, float2>::value) {
        // the band operand's row scale: every G of the band is in exactly one
        // plane, so the blocks of band b together see all of its coefficients
        if (a.rowmax && !a.items) {
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if ((threadIdx.x & 31) == 0 && mx) atomicMax(a.rowmax + b, mx);
        }
    }
    __syncthreads();
    // z (rows of b0): intermediates in b1 then b0; output to the buffer the last stage does not read
    const int rz = fft_last_read(a.Lz);
    C* zo = (rz == 1) ? b0 : b1;
    C* zother = (zo == b0) ? b1 : b0;
    C* Tp = T + ((size_t)b * nxs + p) * n23;
    if constexpr (std::is_same<PL, NoPlan>::value) {
        lines<C, WIDE, PL>(SmemLines<C>{b0, n3p, 1}, SmemLines<C>{zo, n3p, 1}, b1, b0, a.Lz, a.nl_z, n3p, 1, twz,
                           +1);
        __syncthreads();
        // y (columns), last stage straight to T
        lines<C, WIDE, PL>(SmemLines<C>{zo, 1, n3p}, PlaneGlobal<C>{Tp, n3}, zother, zo, a.Ly, a.nl_y, 1, n3p, twy,
                           +1);
    } else {
        constexpr int N = PL::n, NP = PL::n + 1;  // n2 = n3 = N lines per axis
        // z-lines of the rows in use only: the other rows of b0 are zero and
        // stay zero in zo (= b0 for these two-stage plans)
        const int jr = plane_jr ? plane_jr[p] : N;
        if (2 * jr + 1 < N && zo == b0)
            fft_rows_cc<C, PL, NP, 1>(b0, zo, b1, jr, twz, +1);
        else
            fft_lines_cc<C, PL, N>(SmemLinesC<C, NP, 1>{b0}, SmemLinesC<C, NP, 1>{zo}, SmemLinesC<C, NP, 1>{b1}, twz,
                                   +1);
        __syncthreads();
        fft_lines_cc<C, PL, N>(SmemLinesC<C, 1, NP>{zo}, PlaneGlobalC<C, N>{Tp}, SmemLinesC<C, 1, NP>{zother}, twy,
                               +1);
    }
}

// ---- lane-pair plane passes (complex64, compile-time plans) ----------------
// One (plane, band) per block and ONE shared-memory plane of n x (n+1)
// complex64 values (odd row stride: rows and columns conflict-free),
// transformed in place: each z-row and each y-column is owned by one lane
// pair (fftreg::fft_pair: even/odd samples, a half-length register transform
// per lane, one shuffle exchange; the pair is lanes l and l ^ 16, so a
// half-warp reads one run of 16 rows or columns: no bank conflicts, and the
// y-transforms' T accesses are 128-byte runs), so a plane costs three block barriers
// instead of one per Stockham stage.  Blocks are 2n threads rounded up to
// whole warps (160 for n = 72), small enough (one plane, ~100 registers) that
// four or more planes share an SM.
using fftreg::PairPlan;
template <int N> constexpr int pair_threads() { return (2 * N + 31) / 32 * 32; }
template <int N> constexpr int pair_minb() { return N >= 64 ? 4 : (N >= 36 ? 8 : 12); }

// The rows of a plane that hold sphere points, |G_y| <= jr: rows 0..jr and
// n-jr..n-1, or every row when 2 jr + 1 >= n.  row(L) is the L-th of them.
struct PlaneRows {
    int jr, n;
    bool all;
    HPSI_D PlaneRows(int jr_, int n_) : jr(jr_), n(n_), all(2 * jr_ + 1 >= n_) {}
    HPSI_D int count() const { return all ? n : 2 * jr + 1; }
    HPSI_D int row(int L) const { return (all || L <= jr) ? L : L + n - (2 * jr + 1); }
    HPSI_D bool holds(int j) const { return all || j <= jr || j >= n - jr; }
};

// one scatter batch of the G->r plane pass: SB entries per thread, NT apart,
// index loads first, then the psi loads (jk = -1 past the plane's end)
template <int SB, int NT>
HPSI_D void scatter_load(int eb, int e1, const int* __restrict__ ent_ig, const int* __restrict__ ent_jk,
                         const double2* __restrict__ ps, bool want_max, int (&ig)[SB], int (&jk)[SB],
                         double2 (&c)[SB])
{
#pragma unroll
    for (int u = 0; u < SB; ++u) {
        const int e = eb + u * NT;
        ig[u] = e < e1 ? ent_ig[e] : -1;
        jk[u] = e < e1 ? ent_jk[e] : -1;
    }
#pragma unroll
    for (int u = 0; u < SB; ++u) {
        // a G that shares its grid point with a later one (ig < 0) is not
        // scattered, but its coefficient is still a row element of the band operand
        const bool need = jk[u] >= 0 && (ig[u] >= 0 || want_max);
        c[u] = need ? ps[ig[u] & 0x7fffffff] : make_double2(0.0, 0.0);
    }
}

template <typename PL>
__global__ void __launch_bounds__(pair_threads<PL::n>(), pair_minb<PL::n>())
    g2r_planes_pair(LocalArgs a, const double2* __restrict__ psi, float2* __restrict__ T)
{
    constexpr int N = PL::n, NP = N + 1, N23 = N * N, H1 = PairPlan<N>::h1, H2 = PairPlan<N>::h2, H = N / 2;
    constexpr int NT = pair_threads<N>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* pl = reinterpret_cast<float2*>(smem_raw);
    const int p = blockIdx.x;
    int b = blockIdx.y;
    int npw = a.npw, nxs = a.nxs;
    const int *plane_off = a.plane_off, *ent_ig = a.ent_ig, *ent_jk = a.ent_jk, *plane_jr = a.plane_jr;
    if (a.items) {  // batched: the band's item (uniform per block, before any barrier)
        const LocalItem I = a.items[a.band_item[b]];
        if (p >= I.nxs) return;
        b -= I.band0;
        npw = I.npw; nxs = I.nxs;
        plane_off = I.plane_off; ent_ig = I.ent_ig; ent_jk = I.ent_jk; plane_jr = I.plane_jr;
        psi = I.psi;
        T += I.t_off;
    }
    const PlaneRows rows(plane_jr ? plane_jr[p] : N, N);
    const int nrows = rows.count();
    const double2* ps = psi + (size_t)b * npw;
    const int e0 = plane_off[p], e1 = plane_off[p + 1];
    uint32_t mx = 0u;  // float bits of the largest |re|, |im| this thread scattered
    // in batches of SB entries per thread: all index loads, then all psi loads,
    // then the stores, so the two dependent global round trips are paid once
    // per batch, not once per entry; the first batch's loads are issued before
    // the plane buffer is zeroed, which hides the zeroing behind them
    constexpr int SB = 8;
    const bool want_max = a.rowmax && !a.items;
    int eb = e0 + threadIdx.x;
    int ig[SB], jk[SB];
    double2 c[SB];
    scatter_load<SB, NT>(eb, e1, ent_ig, ent_jk, ps, want_max, ig, jk, c);
    // zero the rows in use (the others are never read): one run of the plane
    // buffer, or two (rows 0..jr and N-jr..N-1), in 16-byte stores; a run's
    // ends are rounded outwards to whole float4s, which only touches elements
    // of rows not in use (N is even, so the buffer is a whole number of float4s)
    {
        constexpr int E4 = N * NP / 2;
        const int a1 = rows.all ? E4 : ((rows.jr + 1) * NP + 1) / 2;
        const int b0 = rows.all ? E4 : ((N - rows.jr) * NP) / 2;
        const int cnt = a1 + (E4 - b0);
        float4* z4 = reinterpret_cast<float4*>(pl);
        for (int t = threadIdx.x; t < cnt; t += NT) z4[t < a1 ? t : t - a1 + b0] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    for (;;) {
#pragma unroll
        for (int u = 0; u < SB; ++u) {
            if (jk[u] < 0) continue;
            const float2 v = to_c64(c[u]);
            if (ig[u] >= 0) {
                const int j = jk[u] / N, k = jk[u] - (jk[u] / N) * N;
                pl[j * NP + k] = v;
            }
            mx = max(mx, max(__float_as_uint(v.x) & 0x7fffffffu, __float_as_uint(v.y) & 0x7fffffffu));
        }
        eb += SB * NT;
        if (eb >= e1) break;
        scatter_load<SB, NT>(eb, e1, ent_ig, ent_jk, ps, want_max, ig, jk, c);
    }
    if (a.rowmax && !a.items) {
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0 && mx) atomicMax(a.rowmax + b, mx);
    }
    __syncthreads();
    // lane pair (l, l ^ 16) of warp w: pair index 16 w + (l & 15)
    const int pr = (threadIdx.x >> 5) * 16 + (threadIdx.x & 15);
    const bool odd = (threadIdx.x >> 4) & 1;
    float2 v[H];
    // z (rows in use), G->r, in place; a warp with no row in use skips it
    // (warp-uniform: both lanes of every pair are in the same warp)
    if (__any_sync(0xffffffffu, pr < nrows)) {
        const bool on = pr < nrows;
        float2* row = pl + (on ? rows.row(pr) : 0) * NP;
#pragma unroll
        for (int n = 0; n < H; ++n) v[n] = on ? row[2 * n + odd] : make_float2(0.f, 0.f);
        fftreg::fft_pair<+1, H1, H2>(v, odd);
        if (on) {
#pragma unroll
            for (int m = 0; m < H; ++m) row[m + (odd ? H : 0)] = v[fftreg::split_pos<H1, H2>(m)];
        }
    }
    __syncthreads();
    // y (columns), G->r, straight to T: the even lane holds rows 2n, the odd 2n+1
    {
        const bool on = pr < N;
        const int k = on ? pr : 0;
#pragma unroll
        for (int n = 0; n < H; ++n) {
            const int j = 2 * n + (odd ? 1 : 0);
            v[n] = (on && rows.holds(j)) ? pl[j * NP + k] : make_float2(0.f, 0.f);
        }
        fftreg::fft_pair<+1, H1, H2>(v, odd);
        if (on) {
            float2* Tp = T + ((size_t)b * nxs + p) * N23 + k + (odd ? H * N : 0);
#pragma unroll
            for (int m = 0; m < H; ++m) Tp[(size_t)m * N] = v[fftreg::split_pos<H1, H2>(m)];
        }
    }
}

template <typename PL>
__global__ void __launch_bounds__(pair_threads<PL::n>(), pair_minb<PL::n>())
    r2g_planes_pair(LocalArgs a, const float2* __restrict__ T, const double2* __restrict__ psi,
                    double2* __restrict__ hpsi, const double* __restrict__ kinetic)
{
    constexpr int N = PL::n, NP = N + 1, N23 = N * N, H1 = PairPlan<N>::h1, H2 = PairPlan<N>::h2, H = N / 2;
    constexpr int NT = pair_threads<N>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* pl = reinterpret_cast<float2*>(smem_raw);
    const int p = blockIdx.x;
    int b = blockIdx.y;
    int npw = a.npw, nxs = a.nxs;
    const int *plane_off = a.plane_off, *ent_ig = a.ent_ig, *ent_jk = a.ent_jk, *plane_jr = a.plane_jr;
    if (a.items) {  // batched: the band's item (uniform per block, before any barrier)
        const LocalItem I = a.items[a.band_item[b]];
        if (p >= I.nxs) return;
        b -= I.band0;
        npw = I.npw; nxs = I.nxs;
        plane_off = I.plane_off; ent_ig = I.ent_ig; ent_jk = I.ent_jk; plane_jr = I.plane_jr;
        psi = I.psi; hpsi = I.hpsi; kinetic = I.kinetic;
        T += I.t_off;
    }
    const PlaneRows rows(plane_jr ? plane_jr[p] : N, N);
    const int nrows = rows.count();
    // lane pair (l, l ^ 16) of warp w: pair index 16 w + (l & 15)
    const int pr = (threadIdx.x >> 5) * 16 + (threadIdx.x & 15);
    const bool odd = (threadIdx.x >> 4) & 1;
    float2 v[H];
    // y (columns), r->G, from T; only the rows in use are kept
    {
        const bool on = pr < N;
        const int k = on ? pr : 0;
        const float2* Tp = T + ((size_t)b * nxs + p) * N23 + k + (odd ? N : 0);
#pragma unroll
        for (int n = 0; n < H; ++n) v[n] = on ? Tp[(size_t)(2 * n) * N] : make_float2(0.f, 0.f);
        fftreg::fft_pair<-1, H1, H2>(v, odd);
        if (on) {
#pragma unroll
            for (int m = 0; m < H; ++m) {
                const int j = m + (odd ? H : 0);
                if (rows.holds(j)) pl[j * NP + k] = v[fftreg::split_pos<H1, H2>(m)];
            }
        }
    }
    __syncthreads();
    // z (rows in use), r->G, in place; a warp with no row in use skips it
    if (__any_sync(0xffffffffu, pr < nrows)) {
        const bool on = pr < nrows;
        float2* row = pl + (on ? rows.row(pr) : 0) * NP;
#pragma unroll
        for (int n = 0; n < H; ++n) v[n] = on ? row[2 * n + odd] : make_float2(0.f, 0.f);
        fftreg::fft_pair<-1, H1, H2>(v, odd);
        if (on) {
#pragma unroll
            for (int m = 0; m < H; ++m) row[m + (odd ? H : 0)] = v[fftreg::split_pos<H1, H2>(m)];
        }
    }
    __syncthreads();
    // gather: kinetic*psi + grid/N in FP32, one FP64 add per component into
    // hpsi, or stored to out32 (the tensor-core expansion adds it)
    const double2* ps = psi + (size_t)b * npw;
    double2* hp = hpsi + (size_t)b * npw;
    const int e0 = plane_off[p], e1 = plane_off[p + 1];
    const float inv_n = (float)a.inv_n;
    float2* o32 = (a.out32 && !a.items) ? a.out32 + (size_t)b * npw : nullptr;
    // in batches of GB entries per thread: index loads, then psi / kinetic
    // (and hpsi) loads, then the stores
    constexpr int GB = 4;
    for (int eb = e0 + threadIdx.x; eb < e1; eb += GB * NT) {
        int ig[GB], jk[GB];
#pragma unroll
        for (int u = 0; u < GB; ++u) {
            const int e = eb + u * NT;
            ig[u] = e < e1 ? (ent_ig[e] & 0x7fffffff) : -1;
            jk[u] = e < e1 ? ent_jk[e] : 0;
        }
        double2 c[GB], h[GB];
        double kd[GB];
#pragma unroll
        for (int u = 0; u < GB; ++u) {
            c[u] = ig[u] >= 0 ? ps[ig[u]] : make_double2(0.0, 0.0);
            kd[u] = ig[u] >= 0 ? kinetic[ig[u]] : 0.0;
            h[u] = (ig[u] >= 0 && !o32) ? hp[ig[u]] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < GB; ++u) {
            if (ig[u] < 0) continue;
            const int j = jk[u] / N, k = jk[u] - (jk[u] / N) * N;
            const float2 g = pl[j * NP + k];
            const float2 s = to_c64(c[u]);
            const float kin = d2f_bits(kd[u]);
            const float2 t = make_float2(fmaf(kin, s.x, g.x * inv_n), fmaf(kin, s.y, g.y * inv_n));
            if (o32) {
                o32[ig[u]] = t;
            } else {
                h[u].x += f2d_bits(t.x);
                h[u].y += f2d_bits(t.y);
                hp[ig[u]] = h[u];
            }
        }
    }
}

// x pass: a block owns the x-lines of (j, k0..k0+KT) for BB consecutive bands
// (NL = KT*BB lines, line L = bb*KT + kk, element x at [x*NL + L]); the V tile
// is loaded once per block.  The G->r transform reads the sphere planes of T
// directly (zero for other x) and multiplies by V as it stores; the r->G
// transform stores the sphere planes back into T.
// line L -> (band in block, z-value): KTC > 0 is a compile-time KT
template <int KTC>
HPSI_D int line_band(int L, const FastDiv& ktf)
{
    if constexpr (KTC > 0) return L / KTC;
    else return (int)fdiv((uint32_t)L, ktf);
}

template <typename C, int KTC>
struct XLoad {
    const C* T;
    const int* xpl;      // smem: plane index of x or -1
    size_t plane;        // n2*n3
    size_t base;         // j*n3 + k0
    int nxs, KT, kt, nbb, bb0;
    FastDiv ktf;
    HPSI_D C operator()(int L, int x) const
    {
        const int bb = line_band<KTC>(L, ktf), kk = L - bb * (KTC > 0 ? KTC : KT);
        const int pl = xpl[x];
        if (pl < 0 || bb >= nbb || kk >= kt) return cmake<C>(0, 0);
        return T[((size_t)(bb0 + bb) * nxs + pl) * plane + base + kk];
    }
};

template <typename C, typename V, int KTC>
struct XStoreV {
    C* buf;
    const V* vt;         // smem V tile [x*KT + kk]
    int NL, KT;
    FastDiv ktf;
    HPSI_D void operator()(int L, int x, C v) const
    {
        const int bb = line_band<KTC>(L, ktf), kk = L - bb * (KTC > 0 ? KTC : KT);
        buf[x * NL + L] = cscale(v, (typename Real<C>::type)vt[x * KT + kk]);
    }
};

template <typename C, int KTC>
struct XStore {
    C* T;
    const int* xpl;
    size_t plane, base;
    int nxs, KT, kt, nbb, bb0;
    FastDiv ktf;
    HPSI_D void operator()(int L, int x, C v) const
    {
        const int bb = line_band<KTC>(L, ktf), kk = L - bb * (KTC > 0 ? KTC : KT);
        const int pl = xpl[x];
        if (pl < 0 || bb >= nbb || kk >= kt) return;
        T[((size_t)(bb0 + bb) * nxs + pl) * plane + base + kk] = v;
    }
};

template <typename C, typename V, bool WIDE, bool ENERGY, typename PL, int KTC>
__global__ void __launch_bounds__(256, xpass_min<C, WIDE, PL>()) x_pass(LocalArgs a, int nb, C* __restrict__ T, const V* __restrict__ vloc,
                                              const C* __restrict__ tw_x_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3, KT = a.kt, BB = a.bb, NL = KT * BB;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n1 * NL;
    C* twx = b1 + n1 * NL;
    V* vt = reinterpret_cast<V*>(twx + n1);
    int* xpl = reinterpret_cast<int*>(vt + n1 * KT);
    const int j = blockIdx.y;
    const int k0 = blockIdx.x * KT;
    const int kt = min(KT, n3 - k0);
    int bb0 = blockIdx.z * BB;
    int nxs = a.nxs;
    const int* plane_x = a.plane_x;
    if (a.items) {  // batched: (item, first band) of this band block
        const int2 xb = a.xblk[blockIdx.z];
        const LocalItem I = a.items[xb.x];
        bb0 = xb.y;
        nb = I.nb;
        nxs = I.nxs;
        plane_x = I.plane_x;
        T += I.t_off;
    }
    const int nbb = min(BB, nb - bb0);
    const size_t plane = (size_t)n2 * n3;
    for (int t = threadIdx.x; t < n1; t += blockDim.x) { twx[t] = tw_x_g[t]; xpl[t] = -1; }
    for (int t = threadIdx.x; t < n1 * KT; t += blockDim.x) {
        int x = t / KT, kk = t % KT;
        vt[t] = kk < kt ? vloc[((size_t)x * n2 + j) * n3 + k0 + kk] : (V)0;
    }
    // energy sums: per-line FP64 totals, per-thread partials, and the FP32
    // correction dV = V64 - V of the tile (zero when V is already FP64)
    using R = typename Real<C>::type;
    const int TPL = 256 / NL > 1 ? 256 / NL : 1;  // threads per line in the energy pass
    double* lsum = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(xpl + n1) + 7) & ~static_cast<uintptr_t>(7));
    R* psum = reinterpret_cast<R*>(lsum + 2 * NL);
    float* dvt = reinterpret_cast<float*>(psum + 3 * NL * TPL);
    if constexpr (ENERGY) {
        for (int t = threadIdx.x; t < n1 * KT; t += blockDim.x) {
            int x = t / KT, kk = t % KT;
            float d = 0.f;
            if (a.dv32 && kk < kt) d = a.dv32[((size_t)x * n2 + j) * n3 + k0 + kk];
            dvt[t] = d;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nxs; t += blockDim.x) xpl[plane_x[t]] = t;
    __syncthreads();
    const size_t base = (size_t)j * n3 + k0;
    const XLoad<C, KTC> ld{T, xpl, plane, base, nxs, KT, kt, nbb, bb0, a.kt_f};
    // G->r, times V, into the buffer the last stage does not read
    const int r = fft_last_read(a.Lx);
    C* vo = (r == 1) ? b1 : b0;
    if constexpr (!ENERGY) {
        lines<C, WIDE, PL>(ld, XStoreV<C, V, KTC>{vo, vt, NL, KT, a.kt_f}, b0, b1, a.Lx, a.nl_x, 1, NL, twx, +1);
        __syncthreads();
    } else {
        // psi(r) unscaled; sums of V|psi|^2 and |psi|^2 per line, then psi <- V psi.
        // Each of TPL threads per line accumulates a strided slice of x in the
        // working precision (with the FP64 part of V as dV); the slices are
        // combined in a fixed order, in FP64 or (complex64) compensated FP32.
        lines<C, WIDE, PL>(ld, SmemLines<C>{vo, 1, NL}, b0, b1, a.Lx, a.nl_x, 1, NL, twx, +1);
        __syncthreads();
        for (int t = threadIdx.x; t < NL * TPL; t += blockDim.x) {
            const int L = t % NL, part = t / NL, kk = L % KT;
            R s1 = 0, s1c = 0, s0 = 0;
            for (int x = part; x < n1; x += TPL) {
                const C v = vo[x * NL + L];
                const R w = (R)vt[x * KT + kk];
                const R m = v.x * v.x + v.y * v.y;
                s0 += m;
                s1 += w * m;
                s1c += (R)dvt[x * KT + kk] * m;
                vo[x * NL + L] = cscale(v, w);
            }
            psum[3 * t] = s1;
            psum[3 * t + 1] = s1c;
            psum[3 * t + 2] = s0;
        }
        __syncthreads();
        for (int L = threadIdx.x; L < NL; L += blockDim.x) {
            if constexpr (std::is_same<R, float>::value) {
                // compensated FP32 (two-sum) in part order: GB300's FP64 rate
                // made the FP64 version of this loop a third of the pass
                Sum2f s1, s0;
                for (int part = 0; part < TPL; ++part) {
                    const int t = part * NL + L;
                    s1.add(psum[3 * t]);
                    s1.add(psum[3 * t + 1]);
                    s0.add(psum[3 * t + 2]);
                }
                lsum[2 * L] = f2d_bits(s1.s) + f2d_bits(s1.c);
                lsum[2 * L + 1] = f2d_bits(s0.s) + f2d_bits(s0.c);
            } else {
                double s1 = 0.0, s0 = 0.0;
                for (int part = 0; part < TPL; ++part) {
                    const int t = part * NL + L;
                    s1 += (double)psum[3 * t] + (double)psum[3 * t + 1];
                    s0 += (double)psum[3 * t + 2];
                }
                lsum[2 * L] = s1;
                lsum[2 * L + 1] = s0;
            }
        }
        __syncthreads();
        double* sums = lsum;
        const int nslots = gridDim.x * gridDim.y, slot = blockIdx.y * gridDim.x + blockIdx.x;
        for (int bb = threadIdx.x; bb < nbb; bb += blockDim.x) {
            double s1 = 0.0, s0 = 0.0;
            for (int kk = 0; kk < kt; ++kk) {
                s1 += sums[2 * (bb * KT + kk)];
                s0 += sums[2 * (bb * KT + kk) + 1];
            }
            double* e = a.epart + ((size_t)(a.e_band0 + bb0 + bb) * nslots + slot) * 2;
            e[0] = s1;
            e[1] = s0;
        }
        __syncthreads();
    }
    // r->G, back into the sphere planes of T
    C* vother = (vo == b0) ? b1 : b0;
    const XStore<C, KTC> stT{T, xpl, plane, base, nxs, KT, kt, nbb, bb0, a.kt_f};
    lines<C, WIDE, PL>(SmemLines<C>{vo, 1, NL}, stT, vother, vo, a.Lx, a.nl_x, 1, NL, twx, -1);
}

// Register x pass (complex64, compile-time plans N = N1*N2 on all axes): one
// thread per x-line (band, j, k).  The thread loads the line's sphere planes
// from T (consecutive threads take consecutive (j, k), so every load and
// store of a warp is one coalesced 256-byte access), transforms it G->r in
// registers, multiplies by V (read at the transform's split positions, no
// reordering), transforms it r->G and stores the sphere planes back.  No
// shared memory but the block's plane mask, no barrier inside the line work.
// Blocks never straddle bands (grid.y = band), so the plane set is uniform.
// Resident blocks per SM by line length: three for N >= 64 (168 registers:
// with the packed pair adds of the transforms the 72-point line fits with a
// 20-byte spill, 0.120 -> 0.116 ms on the 64-atom cell; the energy variant
// keeps two blocks and 255 registers), three for 36, four for 24.
//
// ENERGY: after the G->r transform each thread also sums over its line's N
// points V|psi(r)|^2 (+ dV |psi(r)|^2, the FP64 part of V the FP32 table
// misses) and |psi(r)|^2, in four interleaved FP32 partial sums combined in
// FP64; the block adds its lines' sums in FP64 in a fixed order and writes
// one slot per (band, block):
// epart[((e_band0 + band) * gridDim.x + blockIdx.x) * 2 + {0, 1}].
constexpr int XREG_THREADS = 128;
// resident blocks per SM (the register bound): three for N >= 64 without the
// energy sums (168 registers), two with them (255), three for 36, four for 24
constexpr int xreg_minb(int n, bool energy = false) { return n >= 64 ? (energy ? 2 : 3) : (n >= 36 ? 3 : 4); }

// The line work of the register x passes: G->r transform, the V multiply
// (with the energy sums: four interleaved FP32 partials of V|psi(r)|^2 and
// |psi(r)|^2, dV |psi(r)|^2 in a fifth), leaving r->G to the caller.  vp, dvp:
// the line's V and dV (stride N^2; dvp null: none).
template <typename PL, bool ENERGY>
__device__ __forceinline__ void xline_g2r_v(float2 (&v)[PL::n], const float* __restrict__ vp,
                                            const float* __restrict__ dvp, bool valid, float (&a1)[4], float (&a0)[4],
                                            float& ac)
{
    constexpr int N1 = PL::r0, N2 = PL::r1, N = PL::n, N23 = N * N;
    fftreg::fft_nat_to_split<+1, N1, N2>(v);
#pragma unroll
    for (int x = 0; x < N; ++x) {
        const float w = valid ? __ldg(vp + (size_t)x * N23) : 0.f;
        float2& e = v[fftreg::split_pos<N1, N2>(x)];
        if constexpr (ENERGY) {
            // four interleaved FP32 partial sums per line (N/4 terms each);
            // the FP64 part of V the FP32 table misses (dV) in one more
            const float mm = e.x * e.x + e.y * e.y;
            a1[x & 3] += w * mm;
            a0[x & 3] += mm;
            if (dvp && valid) ac += __ldg(dvp + (size_t)x * N23) * mm;
        }
        // rounded product (never fused into the next stage's adds), so that
        // both variants of the kernel give bit-identical hpsi
        e = make_float2(__fmul_rn(e.x, w), __fmul_rn(e.y, w));
    }
}

// one thread's line energy sums of a block of XREG_THREADS lines, added in
// FP64 in a fixed order and written by thread 0 to e[0], e[1]; red: the
// block's scratch (a __syncthreads separates its uses)
__device__ __forceinline__ void xline_energy_block(const float (&a1)[4], const float (&a0)[4], float ac,
                                                   double (&red)[2][XREG_THREADS / 32], double* e)
{
    double t1 = (f2d_bits(a1[0]) + f2d_bits(a1[1])) + (f2d_bits(a1[2]) + f2d_bits(a1[3])) + f2d_bits(ac);
    double t0 = (f2d_bits(a0[0]) + f2d_bits(a0[1])) + (f2d_bits(a0[2]) + f2d_bits(a0[3]));
    for (int o = 16; o > 0; o >>= 1) {
        t1 += __shfl_xor_sync(0xffffffffu, t1, o);
        t0 += __shfl_xor_sync(0xffffffffu, t0, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = t1;
        red[1][threadIdx.x >> 5] = t0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double u1 = 0.0, u0 = 0.0;
        for (int w = 0; w < XREG_THREADS / 32; ++w) {
            u1 += red[0][w];
            u0 += red[1][w];
        }
        e[0] = u1;
        e[1] = u0;
    }
}

template <typename PL, bool ENERGY>
__global__ void __launch_bounds__(XREG_THREADS, xreg_minb(PL::n, ENERGY)) x_pass_reg(LocalArgs a, float2* __restrict__ T,
                                                              const float* __restrict__ vloc)
{
    constexpr int N1 = PL::r0, N2 = PL::r1, N = PL::n, N23 = N * N, W = (N + 31) / 32;
    __shared__ uint32_t msk[W];
    __shared__ double red[2][XREG_THREADS / 32];
    // bands in reverse launch order: the G->r pass wrote the last bands last,
    // so they are the ones still in L2 (the r->G pass then runs forward over
    // the bands written last here)
    int b = a.items ? (int)blockIdx.y : (int)(gridDim.y - 1 - blockIdx.y);
    int nxs = a.nxs;
    const int* plane_x = a.plane_x;
    if (a.items) {  // batched: the band's item (uniform per block)
        const LocalItem I = a.items[a.band_item[b]];
        b -= I.band0;
        nxs = I.nxs;
        plane_x = I.plane_x;
        T += I.t_off;
    }
    if (threadIdx.x < W) msk[threadIdx.x] = 0u;
    __syncthreads();
    for (int t = threadIdx.x; t < nxs; t += blockDim.x) atomicOr(&msk[plane_x[t] >> 5], 1u << (plane_x[t] & 31));
    __syncthreads();
    const int jk = blockIdx.x * XREG_THREADS + threadIdx.x;
    const bool valid = jk < N23;
    if (!ENERGY && !valid) return;
    uint32_t m[W];
#pragma unroll
    for (int w = 0; w < W; ++w) m[w] = valid ? msk[w] : 0u;  // an idle energy thread loads and stores nothing
    float2* line = T + (size_t)b * nxs * N23 + jk;
    float2 v[N];
    {
        const float2* p = line;
#pragma unroll
        for (int x = 0; x < N; ++x) {
            const bool on = (m[x >> 5] >> (x & 31)) & 1u;
            v[x] = on ? __ldcs(p) : make_float2(0.f, 0.f);
            if (on) p += N23;
        }
    }
    float a1[4] = {0.f, 0.f, 0.f, 0.f}, a0[4] = {0.f, 0.f, 0.f, 0.f}, ac = 0.f;
    xline_g2r_v<PL, ENERGY>(v, vloc + jk, (ENERGY && a.dv32) ? a.dv32 + jk : nullptr, valid, a1, a0, ac);
    if constexpr (ENERGY) {
        xline_energy_block(a1, a0, ac, red, a.epart + ((size_t)(a.e_band0 + b) * gridDim.x + blockIdx.x) * 2);
        if (!valid) return;
    }
    fftreg::fft_split_to_nat<-1, N1, N2>(v);
    {
        float2* p = line;
#pragma unroll
        for (int x = 0; x < N; ++x) {
            if ((m[x >> 5] >> (x & 31)) & 1u) {
                __stcs(p, v[x]);
                p += N23;
            }
        }
    }
}

// Density x pass of the register plans (complex64, N in {24, 36, 64, 72}):
// one x-line (j, k) per lane pair (lanes l and l ^ 16; a half-warp takes 16
// consecutive lines, so every load is a 128-byte run), and a group of
// XD_BANDS bands per thread (blockIdx.y).  Per band the pair loads its line's
// sphere planes (even lane the even x, odd lane the odd x), transforms it G->r
// with the lane-pair transform and adds occ_b |psi_b(x)|^2 (the product in
// FP32) to compensated FP32 sums of its 36 outputs; the group's sums go to
// part[group][x][jk] in FP64, and density_groups_kernel adds the groups in
// order into rho: the result does not depend on the launch shape.
constexpr int XD_BANDS = 8, XD_THREADS = 128;

template <typename PL>
__global__ void __launch_bounds__(XD_THREADS, PL::n >= 64 ? 2 : 3)
    x_density_pair(LocalArgs a, int nb, const float2* __restrict__ T, const double* __restrict__ occ,
                   double* __restrict__ part)
{
    constexpr int N = PL::n, N23 = N * N, H1 = fftreg::PairPlan<N>::h1, H2 = fftreg::PairPlan<N>::h2, H = N / 2;
    __shared__ int poff[N];  // plane index of x (-1: no sphere plane), times N^2
    const int nxs = a.nxs;
    for (int t = threadIdx.x; t < N; t += blockDim.x) poff[t] = -1;
    __syncthreads();
    for (int t = threadIdx.x; t < nxs; t += blockDim.x) poff[a.plane_x[t]] = t * N23;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int line = ((blockIdx.x * XD_THREADS + threadIdx.x) >> 5) * 16 + (lane & 15);
    const bool odd = lane >= 16;
    const bool valid = line < N23;
    const int b0 = blockIdx.y * XD_BANDS, b1 = min(nb, b0 + XD_BANDS);
    Sum2f acc[H];
    for (int b = b0; b < b1; ++b) {
        const float2* src = T + (size_t)b * nxs * N23 + (valid ? line : 0);
        float2 v[H];
#pragma unroll
        for (int n = 0; n < H; ++n) {
            const int o = poff[2 * n + (odd ? 1 : 0)];
            v[n] = (valid && o >= 0) ? __ldcs(src + o) : make_float2(0.f, 0.f);
        }
        fftreg::fft_pair<+1, H1, H2>(v, odd);
        const float w = (float)occ[b];
#pragma unroll
        for (int r = 0; r < H; ++r) acc[r].add(w * (v[r].x * v[r].x + v[r].y * v[r].y));
    }
    if (!valid) return;
    double* out = part + (size_t)blockIdx.y * N * N23 + line;
#pragma unroll
    for (int m = 0; m < H; ++m) {
        const Sum2f& q = acc[fftreg::split_pos<H1, H2>(m)];
        out[(size_t)(m + (odd ? H : 0)) * N23] = f2d_bits(q.s) + f2d_bits(q.c);
    }
}

// rho[x][jk] += sum over band groups g (in order) of part[g][x][jk]
__global__ void density_groups_kernel(const double* __restrict__ part, int groups, size_t n, double* __restrict__ rho)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int g = 0; g < groups; ++g) s += part[(size_t)g * n + i];
    rho[i] += s;
}

// Density x pass: a block owns (j, k0..k0+KT) and loops over all bands of the
// chunk in groups of BB: G->r along x, then
//   rho[x][j][k0+kk] += sum_b occ_b |psi_b(x, j, k0+kk)|^2
// with the sum over bands taken in band order in FP64 (one owner thread per
// (x, kk)), so the result does not depend on the launch shape.
template <typename C, bool WIDE>
__global__ void __launch_bounds__(256, WIDE ? (Cfg<C>::x_min + 1) / 2 : Cfg<C>::x_min)
    x_density(LocalArgs a, int nb, const C* __restrict__ T, const double* __restrict__ occ, double* __restrict__ rho,
              const C* __restrict__ tw_x_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3, KT = a.kt, BB = a.bb, NL = KT * BB;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n1 * NL;
    C* twx = b1 + n1 * NL;
    int* xpl = reinterpret_cast<int*>(twx + n1);
    double* acc = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(xpl + n1) + 7) & ~static_cast<uintptr_t>(7));
    const int j = blockIdx.y;
    const int k0 = blockIdx.x * KT;
    const int kt = min(KT, n3 - k0);
    const size_t plane = (size_t)n2 * n3;
    for (int t = threadIdx.x; t < n1; t += blockDim.x) { twx[t] = tw_x_g[t]; xpl[t] = -1; }
    for (int t = threadIdx.x; t < n1 * KT; t += blockDim.x) acc[t] = 0.0;
    __syncthreads();
    for (int t = threadIdx.x; t < a.nxs; t += blockDim.x) xpl[a.plane_x[t]] = t;
    __syncthreads();
    const size_t base = (size_t)j * n3 + k0;
    const int r = fft_last_read(a.Lx);
    C* vo = (r == 1) ? b1 : b0;
    for (int bb0 = 0; bb0 < nb; bb0 += BB) {
        const int nbb = min(BB, nb - bb0);
        const XLoad<C, 0> ld{T, xpl, plane, base, a.nxs, KT, kt, nbb, bb0, a.kt_f};
        lines<C, WIDE, NoPlan>(ld, SmemLines<C>{vo, 1, NL}, b0, b1, a.Lx, a.nl_x, 1, NL, twx, +1);
        __syncthreads();
        for (int t = threadIdx.x; t < n1 * KT; t += blockDim.x) {
            const int x = t / KT, kk = t - (t / KT) * KT;
            double s = acc[t];
            for (int bb = 0; bb < nbb; ++bb) {
                const C v = vo[x * NL + bb * KT + kk];
                s += occ[bb0 + bb] * ((double)v.x * (double)v.x + (double)v.y * (double)v.y);
            }
            acc[t] = s;
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n1 * KT; t += blockDim.x) {
        const int x = t / KT, kk = t - (t / KT) * KT;
        if (kk < kt) rho[((size_t)x * n2 + j) * n3 + k0 + kk] += acc[t];
    }
}

template <typename C, bool WIDE, typename PL>
__global__ void __launch_bounds__(Cfg<C>::plane_threads, WIDE ? 1 : Cfg<C>::plane_min) r2g_planes(LocalArgs a, const C* __restrict__ T, const double2* __restrict__ psi,
                                                  double2* __restrict__ hpsi, const double* __restrict__ kinetic,
                                                  const C* __restrict__ tw_y_g, const C* __restrict__ tw_z_g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n2 = plan_n<PL>(a.n2), n3 = plan_n<PL>(a.n3), n3p = n3 + 1, n23 = n2 * n3, n23p = n2 * n3p;
    C* b0 = reinterpret_cast<C*>(smem_raw);
    C* b1 = b0 + n23p;
    C* twy = b1 + n23p;
    C* twz = twy + n2;
    const int p = blockIdx.x;
    int b = blockIdx.y;
    int npw = a.npw, nxs = a.nxs;
    const int *plane_off = a.plane_off, *ent_ig = a.ent_ig, *ent_jk = a.ent_jk, *plane_jr = a.plane_jr;
    if (a.items) {  // batched: the band's item (uniform per block, before any barrier)
        const LocalItem I = a.items[a.band_item[b]];
        if (p >= I.nxs) return;
        b -= I.band0;
        npw = I.npw; nxs = I.nxs;
        plane_off = I.plane_off; ent_ig = I.ent_ig; ent_jk = I.ent_jk; plane_jr = I.plane_jr;
        psi = I.psi; hpsi = I.hpsi; kinetic = I.kinetic;
        T += I.t_off;
    }
    for (int t = threadIdx.x; t < n2; t += blockDim.x) twy[t] = tw_y_g[t];
    for (int t = threadIdx.x; t < n3; t += blockDim.x) twz[t] = tw_z_g[t];
    __syncthreads();
    // y (columns) straight from T; output into the buffer the last stage does not read
    const int ry = fft_last_read(a.Ly);
    C* yo = (ry == 1) ? b1 : b0;
    C* yother = (yo == b0) ? b1 : b0;
    const int rz = fft_last_read(a.Lz);
    // z intermediates: bufA = yother, bufB = yo; last stage reads yo (rz == 2) or yother (rz == 1) or yo via ld (rz == 0)
    C* zo = (rz == 1) ? yo : yother;
    C* Tp = const_cast<C*>(T) + ((size_t)b * nxs + p) * n23;
    if constexpr (std::is_same<PL, NoPlan>::value) {
        lines<C, WIDE, PL>(PlaneGlobal<C>{Tp, n3}, SmemLines<C>{yo, 1, n3p}, b0, b1, a.Ly, a.nl_y, 1, n3p, twy, -1);
        __syncthreads();
        lines<C, WIDE, PL>(SmemLines<C>{yo, n3p, 1}, SmemLines<C>{zo, n3p, 1}, yother, yo, a.Lz, a.nl_z, n3p, 1, twz,
                           -1);
    } else {
        constexpr int N = PL::n, NP = PL::n + 1;
        fft_lines_cc<C, PL, N>(PlaneGlobalC<C, N>{Tp}, SmemLinesC<C, 1, NP>{yo}, SmemLinesC<C, 1, NP>{b0}, twy, -1);
        __syncthreads();
        // z-lines of the rows in use only: the gather reads no other row
        const int jr = plane_jr ? plane_jr[p] : N;
        if (2 * jr + 1 < N)
            fft_rows_cc<C, PL, NP, 1>(yo, zo, yother, jr, twz, -1);
        else
            fft_lines_cc<C, PL, N>(SmemLinesC<C, NP, 1>{yo}, SmemLinesC<C, NP, 1>{zo}, SmemLinesC<C, NP, 1>{yother},
                                   twz, -1);
    }
    __syncthreads();
    const C* res = zo;
    const double2* ps = psi + (size_t)b * npw;
    double2* hp = hpsi + (size_t)b * npw;
    const int e0 = plane_off[p], e1 = plane_off[p + 1];
    if constexpr (std::is_same<C, float2>::value) {
        // complex64: kinetic*psi + grid/N in FP32 (conversions on the integer
        // pipe), one FP64 add per component into hpsi, or stored to out32
        const float inv_n = (float)a.inv_n;
        float2* o32 = (a.out32 && !a.items) ? a.out32 + (size_t)b * npw : nullptr;
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            int ig = ent_ig[e] & 0x7fffffff;
            int jk = ent_jk[e];
            int j = jk / n3, k = jk - j * n3;
            const float2 g = res[j * n3p + k];
            const float2 s = to_c64(ps[ig]);
            const float kin = d2f_bits(kinetic[ig]);
            const float2 t = make_float2(fmaf(kin, s.x, g.x * inv_n), fmaf(kin, s.y, g.y * inv_n));
            if (o32) {
                o32[ig] = t;  // the tensor-core expansion adds it into hpsi
            } else {
                double2 h = hp[ig];
                h.x += f2d_bits(t.x);
                h.y += f2d_bits(t.y);
                hp[ig] = h;
            }
        }
    } else {
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            int ig = ent_ig[e] & 0x7fffffff;
            int jk = ent_jk[e];
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
    size_t b = sizeof(C) * (2 * (size_t)a.n1 * NL + a.n1) + sizeof(V) * (size_t)a.n1 * a.kt + sizeof(int) * a.n1;
    if (a.epart) {
        // energy pass: line totals (double), per-thread partials, dV tile
        const size_t tpl = 256 / NL > 1 ? 256 / NL : 1;
        b = (b + 7) / 8 * 8 + 2 * sizeof(double) * NL + 3 * sizeof(typename Real<C>::type) * NL * tpl +
            sizeof(float) * (size_t)a.n1 * a.kt;
    }
    return b;
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
    if (csize == 8 && nlmax >= 8 && a->n3 >= 4) {
        // complex64: 4 z-values and a power-of-two band group (<= 16) per block,
        // the shape the batch plans' tuner picks for the 36^3 and 72^3 grids
        a->kt = 4;
        int bb = 1;
        while (bb * 2 <= nlmax / 4 && bb * 2 <= 16) bb *= 2;
        a->bb = bb;
    } else {
        a->kt = nlmax < 8 ? nlmax : 8;
        if (a->kt > a->n3) a->kt = a->n3;
        a->bb = nlmax / a->kt;
        if (a->bb < 1) a->bb = 1;
    }
    a->nl_z = make_fastdiv((uint32_t)a->n2);
    a->nl_y = make_fastdiv((uint32_t)a->n3);
    a->nl_x = make_fastdiv((uint32_t)(a->kt * a->bb));
    a->kt_f = make_fastdiv((uint32_t)a->kt);
}

#define XREG_LAUNCH(PL, G)                                                                    \
    do {                                                                                      \
        if (a.epart) x_pass_reg<PL, true><<<G, XREG_THREADS, 0, st>>>(a, T, vloc);           \
        else x_pass_reg<PL, false><<<G, XREG_THREADS, 0, st>>>(a, T, vloc);                  \
    } while (0)

// the register x pass and the lane-pair plane passes serve the complex64
// compile-time plans
template <typename C, typename PL>
constexpr bool xreg_plan()
{
    return std::is_same<C, float2>::value && !std::is_same<PL, NoPlan>::value;
}

// launch of a lane-pair plane kernel: one n x (n+1) complex64 plane per block
template <typename PL>
constexpr size_t pair_smem()
{
    if constexpr (std::is_same<PL, NoPlan>::value) return 0;
    else return sizeof(float2) * (size_t)PL::n * (PL::n + 1);
}
template <typename PL>
constexpr int pair_block()
{
    if constexpr (std::is_same<PL, NoPlan>::value) return 0;
    else return pair_threads<PL::n>();
}

template <typename C, typename V, bool WIDE, typename PL, int KTC>
static cudaError_t launch_local_t(const LocalArgs& a, int nb, const double2* psi, double2* hpsi, const double* kinetic,
                                  C* T, const V* vloc, const C* twx, const C* twy, const C* twz, cudaStream_t st,
                                  Prof* prof)
{
    const size_t sp = plane_smem<C>(a), sx = xpass_smem<C, V>(a);
    cudaError_t e;
    auto g2r = g2r_planes<C, WIDE, PL>;
    auto r2g = r2g_planes<C, WIDE, PL>;
    auto xp = a.epart ? x_pass<C, V, WIDE, true, PL, KTC> : x_pass<C, V, WIDE, false, PL, KTC>;
    if ((e = cudaFuncSetAttribute(g2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(r2g, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(xp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx))) return e;
    if (a.nxs == 0 || nb == 0) return cudaSuccess;
    dim3 gp(a.nxs, nb);
    const int pt = a.plane_threads > 0 ? a.plane_threads : Cfg<C>::plane_threads;
    const int ptg = a.plane_threads > 0 ? a.plane_threads : Cfg<C>::g2r_threads;
    int h = prof->open(PH_G2R, st);
    if constexpr (xreg_plan<C, PL>()) {
        if (a.psi_in[0] && a.psi_mid > 0 && a.psi_mid < nb) {
            // psi in two band halves: each half of the G->r pass as soon as its bands arrived
            const int m = a.psi_mid;
            LocalArgs a2 = a;
            a2.rowmax = a.rowmax ? a.rowmax + m : nullptr;
            if ((e = cudaStreamWaitEvent(st, a.psi_in[0], 0))) return e;
            g2r_planes_pair<PL><<<dim3(a.nxs, m), pair_block<PL>(), pair_smem<PL>(), st>>>(a, psi, T);
            if ((e = cudaStreamWaitEvent(st, a.psi_in[1], 0))) return e;
            g2r_planes_pair<PL><<<dim3(a.nxs, nb - m), pair_block<PL>(), pair_smem<PL>(), st>>>(
                a2, psi + (size_t)m * a.npw, T + (size_t)m * a.nxs * a.n2 * a.n3);
        } else {
            for (int i = 0; i < 2; ++i)
                if (a.psi_in[i] && (e = cudaStreamWaitEvent(st, a.psi_in[i], 0))) return e;
            g2r_planes_pair<PL><<<gp, pair_block<PL>(), pair_smem<PL>(), st>>>(a, psi, T);
        }
    } else {
        for (int i = 0; i < 2; ++i)
            if (a.psi_in[i] && (e = cudaStreamWaitEvent(st, a.psi_in[i], 0))) return e;
        g2r<<<gp, ptg, sp, st>>>(a, psi, T, twy, twz);
    }
    prof->close(h, st);
    if (a.after_g2r && (e = cudaEventRecord(a.after_g2r, st))) return e;
    h = prof->open(PH_XPASS, st);
    if constexpr (xreg_plan<C, PL>()) {
        XREG_LAUNCH(PL, dim3(ceil_div(PL::n * PL::n, XREG_THREADS), nb));
    } else {
        dim3 gx(ceil_div(a.n3, a.kt), a.n2, ceil_div(nb, a.bb));
        xp<<<gx, 256, sx, st>>>(a, nb, T, vloc, twx);
    }
    prof->close(h, st);
    h = prof->open(PH_R2G, st);
    if constexpr (xreg_plan<C, PL>()) {
        r2g_planes_pair<PL><<<gp, pair_block<PL>(), pair_smem<PL>(), st>>>(a, T, psi, hpsi, kinetic);
    } else {
        r2g<<<gp, pt, sp, st>>>(a, T, psi, hpsi, kinetic, twy, twz);
    }
    prof->close(h, st);
    return cudaGetLastError();
}

template <typename C, typename V, bool WIDE, typename PL, int KTC>
static cudaError_t launch_local_batch_t(const LocalArgs& a, int nbands, int max_nxs, int nxblk, C* T, const V* vloc,
                                        const C* twx, const C* twy, const C* twz, cudaStream_t st)
{
    const size_t sp = plane_smem<C>(a), sx = xpass_smem<C, V>(a);
    cudaError_t e;
    auto g2r = g2r_planes<C, WIDE, PL>;
    auto r2g = r2g_planes<C, WIDE, PL>;
    auto xp = x_pass<C, V, WIDE, false, PL, KTC>;
    if ((e = cudaFuncSetAttribute(g2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(r2g, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(xp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx))) return e;
    if (max_nxs == 0 || nbands == 0 || nxblk == 0) return cudaSuccess;
    const int pt = a.plane_threads > 0 ? a.plane_threads : Cfg<C>::plane_threads;
    dim3 gp(max_nxs, nbands);
    if constexpr (xreg_plan<C, PL>()) g2r_planes_pair<PL><<<gp, pair_block<PL>(), pair_smem<PL>(), st>>>(a, nullptr, T);
    else g2r<<<gp, pt, sp, st>>>(a, nullptr, T, twy, twz);
    if constexpr (xreg_plan<C, PL>()) {
        XREG_LAUNCH(PL, dim3(ceil_div(PL::n * PL::n, XREG_THREADS), nbands));
    } else {
        dim3 gx(ceil_div(a.n3, a.kt), a.n2, nxblk);
        xp<<<gx, 256, sx, st>>>(a, 0, T, vloc, twx);
    }
    if constexpr (xreg_plan<C, PL>())
        r2g_planes_pair<PL><<<gp, pair_block<PL>(), pair_smem<PL>(), st>>>(a, T, nullptr, nullptr, nullptr);
    else r2g<<<gp, pt, sp, st>>>(a, T, nullptr, nullptr, nullptr, twy, twz);
    return cudaGetLastError();
}

// Kernel set of a launch: the wide-radix set, a compile-time two-stage plan
// (complex64, the same plan on all three axes; with KT = 4 also a
// compile-time z-tile in the x pass), or the runtime-plan set.
template <int K> using IntC = std::integral_constant<int, K>;
template <typename C, typename F>
static cudaError_t with_kernels(const LocalArgs& a, F&& f)
{
    if (fft_needs_wide(a.Lx) || fft_needs_wide(a.Ly) || fft_needs_wide(a.Lz))
        return f(std::true_type{}, NoPlan{}, IntC<0>{});
    if constexpr (std::is_same<C, float2>::value) {
        const int id = fft_ct_id(a.Lx);
        if (id != FFT_CT_NONE && fft_ct_id(a.Ly) == id && fft_ct_id(a.Lz) == id) {
            const bool k4 = a.kt == 4;
            switch (id) {
                case FFT_CT_72:
                    return k4 ? f(std::false_type{}, FftPlan2<8, 9>{}, IntC<4>{})
                              : f(std::false_type{}, FftPlan2<8, 9>{}, IntC<0>{});
                case FFT_CT_36:
                    return k4 ? f(std::false_type{}, FftPlan2<9, 4>{}, IntC<4>{})
                              : f(std::false_type{}, FftPlan2<9, 4>{}, IntC<0>{});
                case FFT_CT_24:
                    return k4 ? f(std::false_type{}, FftPlan2<8, 3>{}, IntC<4>{})
                              : f(std::false_type{}, FftPlan2<8, 3>{}, IntC<0>{});
                case FFT_CT_64:
                    return k4 ? f(std::false_type{}, FftPlan2<8, 8>{}, IntC<4>{})
                              : f(std::false_type{}, FftPlan2<8, 8>{}, IntC<0>{});
                default: break;
            }
        }
    }
    return f(std::false_type{}, NoPlan{}, IntC<0>{});
}

template <typename C, typename V>
cudaError_t launch_local_batch(const LocalArgs& a, int nbands, int max_nxs, int nxblk, C* T, const V* vloc,
                               const C* twx, const C* twy, const C* twz, cudaStream_t st)
{
    if (!a.items || a.epart) return cudaErrorInvalidValue;
    if (a.plane_threads > Cfg<C>::plane_threads || a.plane_threads % 32) return cudaErrorInvalidValue;
    return with_kernels<C>(a, [&](auto wide, auto pl, auto ktc) {
        return launch_local_batch_t<C, V, decltype(wide)::value, decltype(pl), decltype(ktc)::value>(
            a, nbands, max_nxs, nxblk, T, vloc, twx, twy, twz, st);
    });
}

template <typename C>
static size_t density_smem(const LocalArgs& a)
{
    const size_t NL = (size_t)a.kt * a.bb;
    size_t b = sizeof(C) * (2 * (size_t)a.n1 * NL + a.n1) + sizeof(int) * a.n1;
    return (b + 7) / 8 * 8 + sizeof(double) * (size_t)a.n1 * a.kt;
}

template <typename C, bool WIDE, typename PL>
static cudaError_t launch_density_t(const LocalArgs& a, int nb, const double2* psi, const double* occ, double* rho,
                                    C* T, const C* twx, const C* twy, const C* twz, cudaStream_t st,
                                    double* part)
{
    const size_t sp = plane_smem<C>(a), sx = density_smem<C>(a);
    cudaError_t e;
    auto g2r = g2r_planes<C, WIDE, PL>;
    auto xd = x_density<C, WIDE>;
    if ((e = cudaFuncSetAttribute(g2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))) return e;
    if ((e = cudaFuncSetAttribute(xd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx))) return e;
    if (a.nxs == 0 || nb == 0) return cudaSuccess;
    const int ptg = a.plane_threads > 0 ? a.plane_threads : Cfg<C>::g2r_threads;
    if constexpr (xreg_plan<C, PL>()) {
        g2r_planes_pair<PL><<<dim3(a.nxs, nb), pair_block<PL>(), pair_smem<PL>(), st>>>(a, psi, T);
        if (part) {
            constexpr int N23 = PL::n * PL::n;
            const int groups = ceil_div(nb, XD_BANDS);
            x_density_pair<PL><<<dim3(ceil_div(ceil_div(N23, 16) * 32, XD_THREADS), groups), XD_THREADS, 0, st>>>(
                a, nb, reinterpret_cast<const float2*>(T), occ, part);
            const size_t n = (size_t)PL::n * N23;
            density_groups_kernel<<<ceil_div((long)n, 256), 256, 0, st>>>(part, groups, n, rho);
            return cudaGetLastError();
        }
    } else {
        g2r<<<dim3(a.nxs, nb), ptg, sp, st>>>(a, psi, T, twy, twz);
    }
    xd<<<dim3(ceil_div(a.n3, a.kt), a.n2), 256, sx, st>>>(a, nb, T, occ, rho, twx);
    return cudaGetLastError();
}

template <typename C>
cudaError_t launch_density(const LocalArgs& a, int nb, const double2* psi, const double* occ, double* rho, C* T,
                           const C* twx, const C* twy, const C* twz, cudaStream_t st, double* part)
{
    if (a.items || a.epart) return cudaErrorInvalidValue;
    return with_kernels<C>(a, [&](auto wide, auto pl, auto) {
        return launch_density_t<C, decltype(wide)::value, decltype(pl)>(a, nb, psi, occ, rho, T, twx, twy, twz, st,
                                                                         part);
    });
}

size_t density_part_bytes(const LocalArgs& a, int nb, size_t csize)
{
    if (csize != sizeof(float2) || local_energy_slots(a, csize) != ceil_div(a.n2 * a.n3, XREG_THREADS)) return 0;
    return (size_t)ceil_div(nb, XD_BANDS) * a.n1 * a.n2 * a.n3 * sizeof(double);
}

int local_energy_slots(const LocalArgs& a, size_t csize)
{
    if (csize == sizeof(float2) && !fft_needs_wide(a.Lx) && !fft_needs_wide(a.Ly) && !fft_needs_wide(a.Lz)) {
        const int id = fft_ct_id(a.Lx);
        if (id != FFT_CT_NONE && fft_ct_id(a.Ly) == id && fft_ct_id(a.Lz) == id)
            return ceil_div(a.n2 * a.n3, XREG_THREADS);  // the register x pass: one slot per block of a band
    }
    return ((a.n3 + a.kt - 1) / a.kt) * a.n2;  // the shared-memory x pass: one slot per (j, k-tile) block
}

size_t local_xpass_smem(const LocalArgs& a, bool fp64)
{
    return fp64 ? xpass_smem<double2, double>(a) : xpass_smem<float2, float>(a);
}

template <typename C, typename V>
cudaError_t launch_local(const LocalArgs& a, int nb, const double2* psi, double2* hpsi, const double* kinetic, C* T,
                         const V* vloc, const C* twx, const C* twy, const C* twz, cudaStream_t st, Prof* prof)
{
    return with_kernels<C>(a, [&](auto wide, auto pl, auto ktc) {
        return launch_local_t<C, V, decltype(wide)::value, decltype(pl), decltype(ktc)::value>(
            a, nb, psi, hpsi, kinetic, T, vloc, twx, twy, twz, st, prof);
    });
}

template cudaError_t launch_local<double2, double>(const LocalArgs&, int, const double2*, double2*, const double*,
                                                   double2*, const double*, const double2*, const double2*,
                                                   const double2*, cudaStream_t, Prof*);
template cudaError_t launch_local<float2, float>(const LocalArgs&, int, const double2*, double2*, const double*,
                                                 float2*, const float*, const float2*, const float2*, const float2*,
                                                 cudaStream_t, Prof*);
template cudaError_t launch_local_batch<double2, double>(const LocalArgs&, int, int, int, double2*, const double*,
                                                         const double2*, const double2*, const double2*, cudaStream_t);
template cudaError_t launch_local_batch<float2, float>(const LocalArgs&, int, int, int, float2*, const float*,
                                                       const float2*, const float2*, const float2*, cudaStream_t);
template cudaError_t launch_density<double2>(const LocalArgs&, int, const double2*, const double*, double*, double2*,
                                             const double2*, const double2*, const double2*, cudaStream_t, double*);
template cudaError_t launch_density<float2>(const LocalArgs&, int, const double2*, const double*, double*, float2*,
                                            const float2*, const float2*, const float2*, cudaStream_t, double*);
