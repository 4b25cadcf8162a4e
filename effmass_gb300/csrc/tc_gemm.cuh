// tc_gemm.cuh — interface of the tcgen05 projector GEMMs (tc_gemm.cu).
#pragma once

#include "kernels.cuh"

// One split operand: hi and lo halves (FP16 or BF16, tc_rows_pad(rows) x ldk
// values in the tiled layout of tc_gemm.cu, ldk a multiple of 32) and the
// per-row factor that undoes its power-of-two scale.
struct TcOperand {
    void* hi = nullptr;
    void* lo = nullptr;
    float* inv_scale = nullptr;
    size_t ldk = 0;
};

struct TcEpilogue {
    float* part;               // mode 0: [splits][M][N] partial sums
    double2* hpsi;             // mode 1: output, [nb][ldh]
    int ldh;
    int nb;
    const float* sa_scale;     // per A row
    const float* sb_scale;     // per B row
    const float2* add32;       // mode 1: optional [nb][ldh] term added with the product
};

// Tables from which the generated-operand variant of the projector GEMMs
// writes its A tiles in shared memory: Pr[p][G] = by[j(p)][G] * sf[a(p)][G],
// scaled by a power of two per row and split like a copied operand.  About
// 22 MB for the 64-atom cell instead of 2 x 342 MB of pre-split matrices.
struct TcGen {
    const float* by = nullptr;       // [nby + 1][ldg] beta_rad(|k+G|) Y_lm(k+G) in FP32, zero for G >= npw
                                     // and in the last row
    const float2* sf = nullptr;      // [natom][ldg] structure factors in complex64, zero for G >= npw
    const int2* rows = nullptr;      // [P rounded up to 16] element offsets (a(p) ldg, j(p) ldg) of
                                     // projector p's sf and by rows; past P (0, zero_off)
    const float* p_scale = nullptr;  // [P] split scale of projector row p (projection operand)
    const float* p_inv = nullptr;    // [P] its inverse
    const float* g_scale = nullptr;  // [ldg] split scale of row G of the transposed operand (expansion)
    const float* g_inv = nullptr;    // [ldg] its inverse
    int P = 0, npw = 0, ldg = 0;     // ldg = npw rounded up to whole 128-row tiles
    int zero_off = 0;                // element offset of the zero by row
};

// Device bytes of the generator tables (P projectors over nby distinct
// (radial function, lm) rows and natom atoms)
size_t tc_gen_bytes(int P, int npw, int nby, int natom);
// Build them in mem (tc_gen_bytes): h_rows[p] = (atom, by row), h_byinfo[j] =
// (radial function, lm index) on the host; beta [nrad][npw], ylm [nlm][npw] and
// sf [natom][npw] the slot's FP64 tables.
cudaError_t tc_build_gen(unsigned char* mem, int P, int npw, const int2* h_rows, const int2* h_byinfo, int nby,
                         int natom, const double* beta, const double* ylm, const double2* sf, bool fp16, TcGen* out,
                         cudaStream_t st);

size_t tc_round_k(size_t k);   // K padded to the K depth of a pipeline stage
int tc_chain_splits(size_t ldk, int chain_k);  // splits that keep every split's K depth <= chain_k
int tc_band_rows(int nb);      // B rows for nb bands (re/im blocks of 128)
size_t tc_rows_pad(size_t rows);  // rows of an operand allocation (whole 128-row tiles)
size_t tc_gemm_smem_bytes();
int tc_proj_splits(int P, int nb, size_t ldk);

// Test hook: poll limit of the MMA issuer's wait for a loaded stage (polls <
// 0: the default, about a second); lowered only to make that wait run out.
cudaError_t tc_set_issue_wait_limit(long polls);

// Gradient operands from the stacked c64 matrices [4P][npw] (Pr, dPr_x, dPr_y,
// dPr_z): the projection operand [4P][2npw] and, per direction alpha, the
// expansion operand [npw][4P] = (Pr^T | dPr_alpha^T) (buffers must be zeroed).
cudaError_t tc_build_grad_operands(const float2* pr4, int P, int npw, bool fp16, TcOperand* proj4, TcOperand* exp3,
                                   float* cmax_scratch, cudaStream_t st);
// Band operand of the projection from psi (complex128 [nb][npw]); rowmax: nb scratch words,
// or, with have_max, the per-band maxima already taken (float bits of max |re|, |im|).
cudaError_t tc_band_operand(const double2* psi, int nb, int npw, bool fp16, TcOperand* B, unsigned* rowmax,
                            cudaStream_t st, bool have_max = false);
// Band operand of the expansion from W (complex64 [P][nb]).
cudaError_t tc_w_operand(const float2* W, int P, int nb, bool fp16, TcOperand* B, unsigned* rowmax, cudaStream_t st);
// W[p][b] = lambda_p * sum_G conj(Pr[p][G]) psi[b][G]  (lam may be null); with e_nl also
// e_nl[b] = sum_p lambda_p |<p|psi_b>|^2 in FP64 (eterm: P*nb doubles of scratch)
// With gen the projector operand is generated from those tables (A then only
// supplies ldk and inv_scale = gen->p_inv).
cudaError_t tc_projection(const TcOperand& A, int P, const TcOperand& B, int nb, int nsplit, bool fp16, float* part,
                          const double* lam, int period, float2* W, int* err, cudaStream_t st, Prof* prof,
                          double* eterm = nullptr, double* e_nl = nullptr, const TcGen* gen = nullptr);
// Row operand [rows][2npw] of a complex128 matrix (psi), for conj(A) B^T GEMMs
cudaError_t tc_rows_operand(const double2* x, int rows, int npw, bool fp16, TcOperand* A, cudaStream_t st);
// out[m][n] = sum_G conj(A[m][G]) B[n][G] in complex128 (B a band operand of nb rows)
cudaError_t tc_gemm_c128(const TcOperand& A, int M, const TcOperand& B, int nb, int nsplit, bool fp16, float* part,
                         double2* out, int* err, cudaStream_t st);
// hpsi[b][G] += sum_p W[p][b] Pr[p][G] (+ add32[b][G] when given, summed in FP32 first)
// (gen as in tc_projection; A.inv_scale = gen->g_inv).  Only the G rows
// [row0, row1) (row0 a multiple of 128; row1 < 0: npw) when given.
cudaError_t tc_expansion(const TcOperand& A, int npw, const TcOperand& B, int nb, bool fp16, double2* hpsi, int* err,
                         cudaStream_t st, Prof* prof, const float2* add32 = nullptr, const TcGen* gen = nullptr,
                         int row0 = 0, int row1 = -1);

// ---- ragged (batched) tensor-core nonlocal term ------------------------------
// One item per (k-point, band block) of a batch plan, nb <= 128 bands.  Band
// operands use the compact row layout: band j's re row at j, its im row at
// nbp + j (nbp = nb rounded up to 16, N = 2 nbp <= 256 rows, tiled like the
// other operands).  All items of a call share P (and so K = tc_round_k(2 P)
// of the expansion).
struct TcRagItem {
    TcGen gen;                   // the k-point's generator tables
    const double2* psi;          // [nb][npw]
    double2* hpsi;               // [nb][npw] (+= the nonlocal term)
    const double* lam;           // [P]
    int nb, nbp, npw;
    int k1t;                     // k-tiles of the projection: tc_round_k(2 npw) / 32
    int per, nz;                 // k-tiles per split, splits (every split holds >= 1 k-tile)
    unsigned char *b1h, *b1l;    // projection band operand, tc_rows_pad(2 nbp) x (32 k1t)
    float* b1s;                  // its row factors [2 nbp]
    float* part;                 // [nz][P][2 nbp] split partials
    float2* W;                   // [P][nb] lambda <p|psi>
    unsigned char *b2h, *b2l;    // expansion band operand, tc_rows_pad(2 nbp) x tc_round_k(2 P)
    float* b2s;                  // [2 nbp]
    unsigned* rowmax;            // [nbp] band maxima scratch
};
int tc_rag_nbp(int nb);          // nb rounded up to 16
// Projection chain of every item: band operands from psi, split-K projection
// GEMM (generated projector tiles), reduction to W, band operands of W.
// bands: (item, band) of every band of the call; rows: (item, j) for j < nbp
// of every item; rowmax_all / n_rowmax: the items' rowmax arrays, contiguous.
cudaError_t tc_rag_project(const TcRagItem* d_items, int n_items, const int2* d_bands, int nbands, const int2* d_rows,
                           int nrows, int P, int k1t_max, int nz_max, bool fp16, unsigned* rowmax_all,
                           size_t n_rowmax, int* err, cudaStream_t st);
// Expansion of every item over its 128-row G tiles (item, tile) in tiles.
cudaError_t tc_rag_expand(const TcRagItem* d_items, const int2* d_tiles, int ntiles, int P, bool fp16, int* err,
                          cudaStream_t st);

