// kernels.cuh — argument blocks and launchers shared between the kernel
// translation units and the C-ABI layer (hpsi_api.cu).
#pragma once

#include "common.cuh"
#include "fft.cuh"

#define HPSI_LMAX 4  // highest angular momentum of a projector (s, p, d, f, g)

#include <vector>

// Phases timed by the optional per-launch CUDA-event profile (hpsi_profile).
enum HpsiPhase {
    PH_BUILD = 0,    // projector build (set-up, lazily on first use of a precision)
    PH_G2R = 1,      // scatter + y/z FFT planes
    PH_XPASS = 2,    // x FFT, V multiply, x FFT
    PH_R2G = 3,      // z/y FFT planes + gather + kinetic
    PH_PROJ = 4,     // projection GEMM (split-K partials)
    PH_REDUCE = 5,   // split reduction * lambda
    PH_EXPAND = 6,   // expansion GEMM
    PH_OTHER = 7,    // gradient kinetic term, velocity GEMMs, conversions
    PH_COUNT = 8
};

// Event pairs around launches; read back and summed by hpsi_profile_read.
struct Prof {
    bool on = false;
    struct Rec { int phase; cudaEvent_t a, b; int kernels; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t take()
    {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    int open(int phase, cudaStream_t st)
    {
        if (!on) return -1;
        Rec r{phase, take(), take(), 1};
        cudaEventRecord(r.a, st);
        recs.push_back(r);
        return (int)recs.size() - 1;
    }
    // kernels: the kernel launches the range holds (its count in hpsi_profile_read)
    void close(int h, cudaStream_t st, int kernels = 1)
    {
        if (h < 0) return;
        recs[h].kernels = kernels;
        cudaEventRecord(recs[h].b, st);
    }
};

// ---- local potential (local.cu) -------------------------------------------
// One k-point (with its block of bands) of a batched local-term launch; all
// pointers on the device.
struct LocalItem {
    const int* plane_x;     // [nxs]
    const int* plane_off;   // [nxs+1]
    const int* ent_ig;      // [npw]
    const int* ent_jk;      // [npw]
    const int* plane_jr;    // [nxs] rows in use of plane p: |G_y| <= plane_jr[p]
    const double* kinetic;  // [npw]
    const double2* psi;     // [nb][npw]
    double2* hpsi;          // [nb][npw], accumulated
    size_t t_off;           // first element of the item's T block [nb][nxs][n2][n3]
    int npw, nxs, nb;
    int band0;              // first band of the item in the batch's band numbering
};

struct LocalArgs {
    int n1, n2, n3;
    int npw;
    int nxs;                // x-planes that hold sphere points
    int kt;                 // z-values per block in the x pass
    int bb;                 // bands per block in the x pass
    double inv_n;           // 1/(n1*n2*n3): the R2G normalisation
    float2* out32;          // complex64 r->G gather: write kinetic*psi + grid/N here
                            // ([nb][npw]) instead of adding it into hpsi (null: add)
    unsigned* rowmax;       // complex64 G->r: per band, atomicMax of the float bits of
                            // |re|, |im| of psi (zeroed before; null: not taken)
    cudaEvent_t after_g2r;  // host side: recorded on the stream after the G->r launch
    cudaEvent_t psi_in[2];  // host side (register-transform plans): psi arrives in two band
    int psi_mid;            // halves [0, psi_mid), [psi_mid, nb); G->r waits per half (null: no split)
    const int* plane_x;     // [nxs] grid x index of plane p
    const int* plane_off;   // [nxs+1] entry range of plane p
    const int* ent_ig;      // [npw] caller-order G index; negative = gather only
    const int* ent_jk;      // [npw] j*n3 + k of the entry
    const int* plane_jr;    // [nxs] rows in use of plane p: |G_y| <= plane_jr[p] (null: all)
    FftLen Lx, Ly, Lz;
    FastDiv nl_z;           // z-lines of a plane: n2
    FastDiv nl_y;           // y-lines of a plane: n3
    FastDiv nl_x;           // x-lines of an x-pass block: kt*bb
    FastDiv kt_f;           // divisor by kt
    // batched launches (items == null for one k-point): the plane kernels run
    // blockIdx.y over all bands of the batch, the x pass blockIdx.z over xblk
    const LocalItem* items;
    const int* band_item;   // [bands] item of each batch band
    const int2* xblk;       // [x-pass band blocks] (item, first band within the item)
    int plane_threads;      // block size of the plane kernels (0: default)
    // band energies (null: off): the x pass adds, per band and (j, k-tile)
    // block, FP64 sums of V|psi(r)|^2 and |psi(r)|^2 of the G->r transform at
    // epart[((e_band0 + band) * nslots + slot) * 2 + {0, 1}]
    double* epart;
    int e_band0;
    const float* dv32;      // for those sums: V64(r) - V(r) of the launch's FP32 V,
                            // the part of the FP64 potential it misses (null: none)
};
// energy slots per band of the x pass that runs for complex size csize (a.kt
// set by local_xpass_shape, a.Lx/Ly/Lz by the caller): one per x-pass block
int local_energy_slots(const LocalArgs& a, size_t csize);

size_t local_smem_bytes(const LocalArgs& a, bool fp64);
// choose kt/bb of the x pass for complex size csize (bytes)
void local_xpass_shape(LocalArgs* a, size_t csize);

template <typename C, typename V>
cudaError_t launch_local(const LocalArgs& a, int nb, const double2* psi, double2* hpsi, const double* kinetic, C* T,
                         const V* vloc, const C* twx, const C* twy, const C* twz, cudaStream_t st, Prof* prof);
// rho[i][j][k] += sum_b occ_b |psi_b(r)|^2 over nb bands (FFT in C; FP64 band
// sums, or on the complex64 register plans compensated FP32 sums per group of
// bands added in FP64, with part: density_part_bytes of scratch, else null)
template <typename C>
cudaError_t launch_density(const LocalArgs& a, int nb, const double2* psi, const double* occ, double* rho, C* T,
                           const C* twx, const C* twy, const C* twz, cudaStream_t st, double* part = nullptr);
// scratch of the register density x pass for nb bands (0: the plan has none)
size_t density_part_bytes(const LocalArgs& a, int nb, size_t csize);
// x-pass line buffer bytes of a given (kt, bb) shape
size_t local_xpass_smem(const LocalArgs& a, bool fp64);
// Batched local term over the items of a.items: nbands = all bands of the
// batch, max_nxs = largest nxs, nxblk = x-pass band blocks (a.kt, a.bb set).
template <typename C, typename V>
cudaError_t launch_local_batch(const LocalArgs& a, int nbands, int max_nxs, int nxblk, C* T, const V* vloc,
                               const C* twx, const C* twy, const C* twz, cudaStream_t st);

// ---- projector build (projectors.cu) --------------------------------------
// Per G: spherical coordinates, trig, Y_lm and its angular gradients.
struct GTabArgs {
    int npw, lmax;
    const double* kvec;     // [npw][3]
    double* q;              // [npw]
    double* trig;           // [4][npw]: sin th, cos th, sin ph, cos ph
    double* ylm;            // [(lmax+1)^2][npw]
    double* yth;            // [(lmax+1)^2][npw] dY/dtheta (may be null)
    double* yph;            // [(lmax+1)^2][npw] (1/sin th) dY/dphi (may be null)
};
cudaError_t launch_gtab(const GTabArgs& a, cudaStream_t st);

// Per (species, projector, G): beta(q) and dbeta/dq with the plane-wave norm.
struct BetaArgs {
    int npw, nrad;          // nrad = sum over species of n_proj
    const double* q;
    const double* tables;   // [nrad][nq_max] raw beta tables
    const double* dtables;  // [nrad][nq_max] raw dbeta tables (may be null)
    const int* rad_nq;      // [nrad]
    const double* rad_dq;   // [nrad]
    int nq_max;
    double norm;            // 1/sqrt(omega)
    double* beta;           // [nrad][npw]
    double* dbeta;          // [nrad][npw] (may be null)
    double* dbeta0;         // [nrad] dbeta at q = 0 (may be null)
};
cudaError_t launch_beta(const BetaArgs& a, cudaStream_t st);

// Per (atom, G): S = exp(-i 2 pi k.tau) * prod_d exp(-i 2 pi g_d tau_d).
struct SfArgs {
    int npw, natom;
    const int* g;           // [npw][3]
    const double* tau;      // [natom][3]
    double kf0, kf1, kf2;
    double2* sf;            // [natom][npw]
};
cudaError_t launch_sf(const SfArgs& a, cudaStream_t st);

// One projector row: atom a, radial function rad (global index), l, m.
struct ProjRow {
    int atom, rad, l, m;
};

// Projector matrices Pr[row][G] = beta*Y*S and, with grad, dPr_alpha rows at
// row offsets (1+alpha)*P.
template <typename C>
cudaError_t launch_assemble(int P, int npw, const ProjRow* rows, const double* beta, const double* dbeta,
                            const double* dbeta0, const double* q, const double* trig, const double* ylm,
                            const double* yth, const double* yph, const double2* sf, bool grad, C* out,
                            size_t ld, cudaStream_t st);

// ---- SIMT complex GEMMs (gemm.cu) -----------------------------------------
// Projection, split over K: part[s][m][n] = sum_{k in split s} conj(A[m][k]) * B[n][k]
// split count of a projection GEMM: every SM busy, at least 64 of K per split
int proj_gemm_splits(int M, int N, int K);
template <typename TA, typename TB, typename Acc>
cudaError_t launch_proj_gemm(int M, int N, int K, const TA* A, size_t lda, const TB* B, size_t ldb, Acc* part,
                             int nsplit, cudaStream_t st);
// W[m][n] = scale[m] * sum_s part[s][m][n]   (scale may be null -> 1)
template <typename Acc, typename CW>
cudaError_t launch_reduce_splits(int M, int N, int nsplit, const Acc* part, const double* scale, int scale_period,
                                 CW* W, size_t ldw, cudaStream_t st);
// Expansion: out[n][k] += sum_m W[m][n] * A[m][k]   (out is complex128)
template <typename C>
cudaError_t launch_expand_gemm(int M, int N, int K, const C* W, size_t ldw, const C* A, size_t lda, double2* out,
                               size_t ldo, cudaStream_t st);
// out[i] = from_c128(in[i])
template <typename C>
cudaError_t launch_convert(size_t n, const double2* in, C* out, cudaStream_t st);

// ---- ragged batched SIMT GEMMs (bgemm.cu) ----------------------------------
// One k-point of a batched nonlocal launch; all pointers on the device.
struct BGemmItem {
    const void* pr;        // [P][npw] projector matrix (complex C of the launch)
    const double2* psi;    // [nb][npw]
    double2* hpsi;         // [nb][npw], accumulated
    const double* lam;     // [P]
    size_t part_off;       // first element of the item's partials [nsplit][P][nb]
    size_t w_off;          // first element of the item's reduced W [P][nb]
    int nb, npw;
};

int bgemm_tile_count();
void bgemm_tile_shape(int tile, int* tm, int* tn);
template <typename C, typename Acc>
cudaError_t launch_bproj(int P, const BGemmItem* items, int n_items, int nb_max, int nsplit, int tile, Acc* part,
                         cudaStream_t st);
template <typename C, typename Acc>
cudaError_t launch_bexp(int P, const BGemmItem* items, int n_items, int nb_max, int npw_max, int nsplit, int tile,
                        const Acc* part, C* W, cudaStream_t st);

// ---- FP64 band-energy reductions (energy.cu) -------------------------------
// per band, chunked partial sums of kinetic |psi|^2 and |psi|^2 over G (kin_norm_words(nb) doubles)
cudaError_t launch_kin_norm(int npw, int nb, const double2* psi, const double* kinetic, double* out, cudaStream_t st);
int kin_norm_words(int nb);
// out[2b], out[2b+1] = the x pass's V|psi(r)|^2 and |psi(r)|^2 sums of band b
cudaError_t launch_local_sums(int nb, int nslots, const double* epart, double* out, cudaStream_t st);
// out[b] = sum_p lam_p |sum_s part[s][p][b]|^2 (SIMT projection partials)
template <typename Acc>
cudaError_t launch_nl_energy(int P, int nb, int nsplit, const Acc* part, const double* lam, double* out,
                             cudaStream_t st);
// e[b] = kinetic + S1/S0 * norm + nonlocal (kn from launch_kin_norm; enl may be null)
cudaError_t launch_energy_combine(int nb, const double* kn, const double* loc, const double* enl, double* e,
                                  cudaStream_t st);
// d[b] = Re <psi_b|h_b>;  e[b] = after[b] - before[b]
cudaError_t launch_band_dot(int npw, int nb, const double2* psi, const double2* h, double* d, cudaStream_t st);
cudaError_t launch_band_sub(int nb, const double* after, const double* before, double* e, cudaStream_t st);
// S[n][a][b] = sum_{m != n, |E_n - E_m| > tol} Re(M_a[n][m] M_b[m][n]) / (E_n - E_m), n < n_low;
// skipped[n] = pairs within tol (skipped may be null)
cudaError_t launch_kp_sums(int nb, int n_low, const double2* M, const double* E, double tol, double* S, int* skipped,
                           cudaStream_t st);

// ---- band-batched FP64 vector kernels of the Sternheimer CG (sternheimer.cu) ----
// vectors are [nb][n] complex128; scalars one per band
cudaError_t launch_bdot(int n, int nb, const double2* x, const double2* y, double* d, cudaStream_t st);
// y_b += asign * alpha_b x_b (alpha null: 1)
cudaError_t launch_baxpy(int n, int nb, const double* alpha, double asign, const double2* x, double2* y,
                         cudaStream_t st);
// y_b = asign * alpha_b x_b + beta_b y_b
cudaError_t launch_baxpby(int n, int nb, const double* alpha, double asign, const double2* x, const double* beta,
                          double2* y, cudaStream_t st);
// y_b += scale * e_b x_b
cudaError_t launch_bscale_add(int n, int nb, const double* e, double scale, const double2* x, double2* y,
                              cudaStream_t st);
// z_b(G) = r_b(G) / (max(kin(G) - e_b, 0) + tau)
cudaError_t launch_bprec(int n, int nb, const double* kin, const double* e, double tau, const double2* r, double2* z,
                         cudaStream_t st);
// out_b = active_b && den_b > 0 ? num_b / den_b : 0
cudaError_t launch_bratio(int nb, const double* num, const double* den, const int* active, double* out,
                          cudaStream_t st);

// ---- radial beta(q) / dbeta(q)/dq tables (tables.cu) -------------------------
int beta_table_nq(double dq, double q_max);
// nmax[p] = points of projector p after trimming its trailing zeros
cudaError_t launch_trim(int nr, int np, const double* beta, int* nmax, cudaStream_t st);
cudaError_t launch_beta_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                               const int* nmax, const double* beta, double dq, int nq, double* bq, double* dbq,
                               cudaStream_t st);
// G-sphere of a k-point: counts per g1-plane, then the points in (g1, g2, g3) order
// (B: reciprocal vectors as rows, host array; kf: k in reciprocal coordinates, host)
cudaError_t launch_gs_count(const double* B, const double* kf, double ecut, int gmax, int* counts, cudaStream_t st);
cudaError_t launch_gs_write(const double* B, const double* kf, double ecut, int gmax, const int* offsets, int* g,
                            double* kvec, double* kinetic, cudaStream_t st);

// ---- projector second derivatives for the Hessian (hessian.cu) ---------------
// f[t][p][iq]: F0, F1, F3 radial tables of the projectors (t = 0, 1, 2)
cudaError_t launch_hess_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                               const int* nmax, const double* beta, double dq, int nq, double* f, cudaStream_t st);
// d2[c][row][g], c = xx, yy, zz, xy, xz, yz; ftabs[rad][3][nq]
template <typename C>
cudaError_t launch_hess_assemble(int P, int npw, const ProjRow* rows, const double* ftabs, int nq, double dq,
                                 double inv_sqrt_omega, const double* kvec, const double2* sf, C* d2, cudaStream_t st);
cudaError_t launch_add(size_t n, const double2* x, double2* y, cudaStream_t st);
